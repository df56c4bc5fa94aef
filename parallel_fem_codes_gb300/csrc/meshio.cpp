// Mesh files of the reference, read on the host so that a single-GPU run
// needs neither the partitioner nor its rank files.
//
// * Global mesh (Mesh_Generator/Structured_Mesh/meshGenerator.c:184-209):
//     nnodes
//     x y f_0 ... f_{ndof-1}        one line per node; f_k = 1 free, 0 prescribed
//     nel
//     v0 v1 v2 [-1]                  one line per element (-1 when ndof > 1)
//   Equations are numbered over the free dofs in node order (node I, dof k),
//   which is the numbering a one-rank run of the partitioner starts from;
//   the library applies its local RCM on top when asked (fg_system_create).
// * One-rank partition file (SST/Preprocess.c:127-168, written by
//   Parallel_Preprocess/Preprocess.c:277-320):
//     nnodes
//     x y {Type [Send invP_id]} per dof    Send and invP_id only when Type != 0
//     nel
//     v0 v1 v2
//   Type 1 is a free dof of this rank; Types 2 and 3 (dofs owned by the
//   neighbouring ranks) do not occur in a one-rank file and are refused.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "fg_internal.h"
#include "../../include/femgpu.h"

using namespace fg;

namespace {

struct MeshBuf {
    int nnodes = 0, nel = 0, neq = 0;
    std::vector<double> x, y;
    std::vector<int> type, invp, ien;
};

int parse(const char *path, int ndof, bool rank_file, MeshBuf &m)
{
    FILE *f = std::fopen(path, "r");
    if (!f) { set_error(std::string("cannot open mesh file ") + path); return FG_ERR_ARG; }
    auto bad = [&](const char *what) {
        std::fclose(f);
        set_error(std::string("mesh file ") + path + ": " + what);
        return FG_ERR_ARG;
    };
    if (std::fscanf(f, "%d", &m.nnodes) != 1 || m.nnodes < 0) return bad("node count");
    m.x.resize(m.nnodes);
    m.y.resize(m.nnodes);
    m.type.assign((size_t)m.nnodes * ndof, 0);
    m.invp.assign((size_t)m.nnodes * ndof, -1);
    std::vector<int> seen;
    for (int i = 0; i < m.nnodes; ++i) {
        if (std::fscanf(f, "%lf %lf", &m.x[i], &m.y[i]) != 2) return bad("node coordinates");
        for (int k = 0; k < ndof; ++k) {
            int t = 0;
            if (std::fscanf(f, "%d", &t) != 1) return bad("node flags");
            const size_t q = (size_t)i * ndof + k;
            if (!rank_file) {
                if (t != 0 && t != 1) return bad("node flag other than 0 or 1");
                m.type[q] = t;
                if (t) m.invp[q] = m.neq++;
            } else {
                if (t == 0) continue;
                int send = 0, id = 0;
                if (std::fscanf(f, "%d %d", &send, &id) != 2) return bad("Send / invP_id");
                if (t != 1) return bad("dof owned by another rank (a one-rank file is expected)");
                m.type[q] = 1;
                m.invp[q] = id;
                ++m.neq;
            }
        }
    }
    if (rank_file) {           // invP_id must number the free dofs 0 .. neq-1 once each
        seen.assign(m.neq, 0);
        for (int id : m.invp)
            if (id >= 0) {
                if (id >= m.neq || seen[id]++) return bad("invP_id is not a numbering of the free dofs");
            }
    }
    if (std::fscanf(f, "%d", &m.nel) != 1 || m.nel < 0) return bad("element count");
    m.ien.resize((size_t)m.nel * 3);
    for (int e = 0; e < m.nel; ++e) {
        for (int v = 0; v < 3; ++v) {
            if (std::fscanf(f, "%d", &m.ien[(size_t)e * 3 + v]) != 1) return bad("element vertices");
            const int nv = m.ien[(size_t)e * 3 + v];
            if (nv < 0 || nv >= m.nnodes) return bad("element vertex out of range");
        }
        if (!rank_file && ndof > 1) {
            int tag = 0;
            if (std::fscanf(f, "%d", &tag) != 1) return bad("element tag");
        }
    }
    std::fclose(f);
    return FG_OK;
}

int deliver(const MeshBuf &m, fg_mesh_info *info, double *x, double *y, int *type, int *invp, int *ien)
{
    info->nnodes = m.nnodes;
    info->nel = m.nel;
    info->neq = m.neq;
    if (x) std::copy(m.x.begin(), m.x.end(), x);
    if (y) std::copy(m.y.begin(), m.y.end(), y);
    if (type) std::copy(m.type.begin(), m.type.end(), type);
    if (invp) std::copy(m.invp.begin(), m.invp.end(), invp);
    if (ien) std::copy(m.ien.begin(), m.ien.end(), ien);
    return FG_OK;
}

}  // namespace

extern "C" {

int fg_mesh_read(const char *path, int ndof, fg_mesh_info *info, double *x, double *y, int *type, int *invp,
                 int *ien)
{
    if (!path || !info) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (ndof < 1 || ndof > 4) { set_error("ndof must be in [1, 4]"); return FG_ERR_ARG; }
    MeshBuf m;
    int r = parse(path, ndof, false, m);
    return r ? r : deliver(m, info, x, y, type, invp, ien);
}

int fg_mesh_read_rank(const char *path, int ndof, fg_mesh_info *info, double *x, double *y, int *type, int *invp,
                      int *ien)
{
    if (!path || !info) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (ndof < 1 || ndof > 4) { set_error("ndof must be in [1, 4]"); return FG_ERR_ARG; }
    MeshBuf m;
    int r = parse(path, ndof, true, m);
    return r ? r : deliver(m, info, x, y, type, invp, ien);
}

// Paraview output, one writer for the drivers' Paraview_Output.c files:
//   SST  01_CommonFiles/Paraview_Output.c:22-111   "solucao", points (x, y, u)
//   Euler 01_CommonFiles/Paraview_Output.c:61-114  Density, Temperature, Pressure
//   NS   01_CommonFiles/Paraview_Output.c:83-134   Velocity (3 components), Pressure
// an ASCII VTK UnstructuredGrid of the triangles (cell type 5, offsets 3(e+1))
// with the given point data in order; z lifts the points (the transport
// drivers' 3-D view) or is NULL for z = 0.  A 2-component field is written
// with a third component 0, as the NS writer writes the velocity.
int fg_write_vtu(const char *path, int nnodes, int nel, const double *x, const double *y, const int *ien,
                 int nfields, const fg_vtu_field *fields, const double *z)
{
    if (!path || !x || !y || !ien || (nfields > 0 && !fields)) { set_error("NULL argument"); return FG_ERR_ARG; }
    if (nnodes < 0 || nel < 0 || nfields < 0) { set_error("invalid sizes"); return FG_ERR_ARG; }
    for (int k = 0; k < nfields; ++k)
        if (!fields[k].name || !fields[k].values || fields[k].ncomp < 1 || fields[k].ncomp > 3) {
            set_error("field " + std::to_string(k) + ": a name, values and 1..3 components are required");
            return FG_ERR_ARG;
        }
    for (size_t q = 0; q < (size_t)nel * 3; ++q)
        if (ien[q] < 0 || ien[q] >= nnodes) { set_error("element vertex out of range"); return FG_ERR_ARG; }
    FILE *f = std::fopen(path, "w");
    if (!f) { set_error(std::string("cannot open ") + path + " for writing"); return FG_ERR_ARG; }
    std::fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"BigEndian\">\n");
    std::fprintf(f, "\t<UnstructuredGrid>\n");
    std::fprintf(f, "\t\t<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", nnodes, nel);
    std::fprintf(f, "\t\t\t<PointData Scalars=\"scalars\">\n");
    for (int k = 0; k < nfields; ++k) {
        const fg_vtu_field &fd = fields[k];
        const int nc = fd.ncomp;
        if (nc == 1) {
            std::fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" Name=\"%s\" Format=\"ascii\">\n", fd.name);
            for (int i = 0; i < nnodes; ++i) std::fprintf(f, "\t\t\t\t   %.12f\n", fd.values[i]);
        } else {
            std::fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"3\" Format=\"ascii\">\n",
                         fd.name);
            for (int i = 0; i < nnodes; ++i) {
                const double *v = fd.values + (size_t)i * nc;
                std::fprintf(f, "\t\t\t\t   %.12f   %.12f   %.12f\n", v[0], v[1], nc == 3 ? v[2] : 0.0);
            }
        }
        std::fprintf(f, "\t\t\t\t</DataArray>\n");
    }
    std::fprintf(f, "\t\t\t</PointData>\n\t\t\t<Points>\n");
    std::fprintf(f, "\t\t\t\t<DataArray type=\"Float32\" NumberOfComponents=\"3\" Format=\"ascii\">\n");
    for (int i = 0; i < nnodes; ++i)
        std::fprintf(f, "\t\t\t\t   %.12f\t%.12f\t%.12f\n", x[i], y[i], z ? z[i] : 0.0);
    std::fprintf(f, "\t\t\t\t</DataArray>\n\t\t\t</Points>\n\t\t\t<Cells>\n");
    std::fprintf(f, "\t\t\t\t<DataArray type=\"Int32\" Name=\"connectivity\" Format=\"ascii\">\n");
    for (int e = 0; e < nel; ++e)
        std::fprintf(f, "\t\t\t\t   %d\t%d\t%d\n", ien[3 * (size_t)e], ien[3 * (size_t)e + 1], ien[3 * (size_t)e + 2]);
    std::fprintf(f, "\t\t\t\t</DataArray>\n\t\t\t\t<DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n");
    for (int e = 0; e < nel; ++e) std::fprintf(f, "\t\t\t\t   %d\n", (e + 1) * 3);
    std::fprintf(f, "\t\t\t\t</DataArray>\n\t\t\t\t<DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n");
    for (int e = 0; e < nel; ++e) std::fprintf(f, "\t\t\t\t   %d\n", 5);
    std::fprintf(f, "\t\t\t\t</DataArray>\n\t\t\t</Cells>\n\t\t</Piece>\n\t</UnstructuredGrid>\n</VTKFile>\n");
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    if (!ok) { set_error(std::string("write error on ") + path); return FG_ERR_ARG; }
    return FG_OK;
}

}  // extern "C"
