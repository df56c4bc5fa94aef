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

}  // extern "C"
