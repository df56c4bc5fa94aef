// Internal declarations shared by the host set-up code and the CUDA
// translation units of libfemgpu.  Not part of the public ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace fg {

// ------------------------------------------------------------ error text
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define FG_CUDA(call)                                                        \
    do {                                                                     \
        cudaError_t fg_e_ = (call);                                          \
        if (fg_e_ != cudaSuccess) return ::fg::cuda_fail(fg_e_, #call);      \
    } while (0)

// ------------------------------------------------------------ host topology
// Everything the device layout needs, computed once per mesh on the host.
struct Topology {
    int nnodes = 0, nel = 0, ndof = 1, S = 3, n = 0;
    std::vector<int> ien;        // nel*3, reference element order
    std::vector<int> type;       // nnodes*ndof
    std::vector<int> invp;       // nnodes*ndof, reference equation numbers
    std::vector<int> lm;         // nel*S, reference numbering (Fill_LM), sink = n
    std::vector<int> perm, iperm;// n+1: internal dof i holds reference dof perm[i]
    int band_before = 0, band_after = 0, nnz = 0;
    std::vector<int> colour;     // nel, reference element order
    int ncol = 0;
    std::vector<int> eorder;     // internal element position -> reference element
    std::vector<int> epos;       // reference element -> internal position
    std::vector<int> cptr;       // ncol+1, internal element ranges per colour
    // dof incidence (internal dofs; entries pos*16 + local row), ordered by
    // reference element index, for order-faithful gathers
    std::vector<int> dinc_ptr, dinc;
    // node incidence (entries pos*4 + vertex), ordered by reference element
    std::vector<int> ninc_ptr, ninc;
    std::vector<int> node_dof;   // nnodes*ndof: internal dof or n (sink)
    // patch layout of the matvec: the elements with a free dof, in internal
    // order, cut into patches of at most kPatchElems; inside a patch the
    // elements are grouped by a local colouring
    int npatch = 0, npcol = 0, maxdof = 0, nel_active = 0;
    std::vector<int> pt_elem;    // npatch+1 element offsets (internal positions)
    std::vector<int> pt_dof;     // npatch+1 offsets into dofs
    std::vector<unsigned short> pt_col;  // npatch * kPatchColStride local colour offsets
    std::vector<int> dofs;       // patch-local dof -> internal dof, bit 31 = shared with another patch
    std::vector<unsigned short> lm16;    // nel*S local indices (internal order), 0xFFFF = sink
    // x segment of each patch: its dofs lie in [xlo, xlo + xlen) (xlo and
    // xlen multiples of 8, xlen <= kPatchXCap); lmx16: per element vertex
    // its dof's position in that segment (0xFFFF = sink), for the matvec
    // that copies the segment whole instead of gathering x dof by dof
    std::vector<int> pt_xlo, pt_xlen;
    std::vector<unsigned short> lmx16;
    // 3x3: per patch one 16-byte aligned index blob (x-segment positions
    // [3][W], dof list, incidence lists) at byte offset pt_boff[p]
    std::vector<long long> pt_boff;
    std::vector<unsigned char> blob;
    std::vector<int> pc_ptr, pc_list;    // patches grouped by patch colour
    // per-patch incidence lists: for patch p, at incl[pt_inc[p]] the list
    // starts (pnd + 1 entries) of each local dof, then the staged product
    // positions (row * patch_elems(S) + element) that add into it, in
    // element order; both parts padded to 8 entries (16-byte copies)
    std::vector<int> pt_inc;
    std::vector<unsigned short> incl;
};

// Assembled CSR form of a system (csr_Initialization.c), rows and columns
// in the internal (RCM) numbering, which is the reference's CSR numbering.
struct CsrTopology {
    int n = 0, nnz = 0;
    std::vector<int> ia, ja, diag;       // diag[i]: slot of the diagonal of row i
    std::vector<int> inc_ptr, inc;       // slot -> contributions pos*256 + a*16 + b, reference element order
    std::vector<int> fwd_chunks, bwd_chunks;  // row chunk starts in solve order (32 rows each)
};
int build_csr(const Topology &t, CsrTopology &c);

constexpr int kPatchElems = 1024;      // largest matvec patch (3x3 blocks)
// Elements per matvec patch for S x S blocks (a multiple of 32).  The
// matvec stages every element's S products of a patch in shared memory, so
// larger blocks use smaller patches (a single large mesh then also gets
// more patches, enough to fill the GPU).
// (FG_MV_PE3 ... FG_MV_PE12: compile-time tuning constants.)
#ifndef FG_MV_PE3
#define FG_MV_PE3 1024
#endif
#ifndef FG_MV_PE6
#define FG_MV_PE6 256
#endif
#ifndef FG_MV_PE9
#define FG_MV_PE9 256
#endif
#ifndef FG_MV_PE12
#define FG_MV_PE12 256
#endif
__host__ __device__ constexpr int patch_elems(int S)
{
    return S <= 3 ? FG_MV_PE3 : S <= 6 ? FG_MV_PE6 : S <= 9 ? FG_MV_PE9 : FG_MV_PE12;
}
__host__ __device__ constexpr int round4(int v) { return (v + 3) & ~3; }
// Shared-memory layout of one matvec CTA (bytes).  S x S blocks, S > 3: x
// and y of the patch's dofs (round4(maxdof) each), the staged products
// [S][PE] and the staged 16-bit local indices [S][PE].  3x3 blocks: x, the
// staged products and the patch's incidence lists (ic: up to maxdof + 8 +
// 3 PE 16-bit entries, 16-byte aligned).
struct MvSmem {
    size_t xs, ys, ye, ls, ic, total;
    __host__ __device__ MvSmem(int S, int maxdof, int w)
    {
        const size_t PE = patch_elems(S), md = round4(maxdof > 0 ? maxdof : 1);
        xs = 0;
        if (S == 3) {
            ys = ls = 0;
            ye = md * w;
            ic = (ye + (size_t)S * PE * w + 15) / 16 * 16;
            total = ic + 2 * ((md + 8 + (size_t)S * PE + 7) / 8 * 8);
        } else {
            ys = md * w;
            ye = 2 * md * w;
            ls = ye + (size_t)S * PE * w;
            ic = 0;
            total = ls + (size_t)S * PE * 2;
        }
    }
};
inline size_t mv_smem_bytes(int S, int maxdof, int w) { return MvSmem(S, maxdof, w).total; }
constexpr int kPatchXCap = 1792;       // largest x segment of a 3x3 patch (entries)
constexpr int kPatchMaxLocalColours = 16;
constexpr int kPatchColStride = kPatchMaxLocalColours + 1;

int build_topology(Topology &t, int nnodes, int nel, int ndof, const int *ien,
                   const int *type, const int *invp, int neq, int reorder);

// Reverse Cuthill-McKee with the tie-breaking of the reference
// (00_CommonFiles/Reordering/symrcm.c); IA/JA row-sorted, symmetric or not.
void symrcm(int n, const int *IA, const int *JA, int *perm);
int matrix_bandwidth(int n, const int *IA, const int *JA);

// ------------------------------------------------------------ device layout
constexpr int kMaxColours = 64;
constexpr int kElemChunk = 1024;   // elements per matvec work item
constexpr int kMaxParts = 1024;    // dof parts (reduction partials) per system
// Dofs per part of the Krylov dof kernels, chosen per batch (unless the
// autotuner cached a choice): 2 sqrt(batch dofs), rounded to the nearest
// power of two, within [kPartMin, kPartMax], so small systems spread over
// many SMs and large batches keep the per-part overhead low.  Fitted to measured optima on GB300 (one
// restart cycle): 16k dofs -> 256-dof parts, 65k -> 512, 147k -> 1024,
// 3.1M (one NS system) -> ~3k, the 24.8M-dof served batch -> 8k-16k.
constexpr int kPartMin = 256;
constexpr int kPartMax = 16384;
constexpr int kThreads = 256;

struct SysState {
    int live;          // system still being solved
    int in_cycle;      // Arnoldi continues in the current cycle
    int steps;         // Arnoldi steps in the current cycle
    int cycles;        // completed cycles
    int iterations;    // total Arnoldi steps
    int converged;
    int status;        // FG_OK / FG_ERR_*
    int first;         // next cycle is the first
    double rho, eps, normb, r0, target, true_res, fnorm, hn;
};

// Per-system descriptor read by every kernel (device memory).
struct SysDev {
    int n, n_pad, nel, nel_pad, S, ndof, ncol, nparts, nnodes;
    int kmax, lmax, mixed, precond;
    int vhalf;                 // basis stored in FP16, scaled by vsc (a power of two)
    float vsc, vsci;           // sigma ~ sqrt(n) and 1 / sigma (1 without vhalf)
    double tol, inner_tol;
    const int *lm;             // [S][nel_pad] internal dofs
    const unsigned short *lm16;// [S][nel_pad] patch-local indices (0xFFFF = sink)
    const int *pt_elem, *pt_dof, *dofs;
    const unsigned short *pt_col;
    const int *pt_inc;                 // per-patch incidence lists (3x3 matvec)
    const unsigned short *incl;
    const unsigned char *blob;         // per-patch index blobs (3x3 bulk-copy matvec)
    int maxdof;
    // assembled CSR operator and ILU(0) (op == 1)
    int op, csr_w;
    const int *csr_ia, *csr_ja, *csr_diag;
    const int *lu_ia, *lu_ja, *lu_dg;    // ILU(p) factor pattern
    const double *AA64, *LU64, *dinv64;
    const float *AA32, *LU32, *dinv32;
    void *ilu_tmp;             // forward-substitution output (T, n_pad)
    const int *ilu_ford, *ilu_bord;      // rows in forward / backward level order
    const int2 *ilu_fpass, *ilu_bpass;   // passes (start, rows) of those orders
    int ilu_P;                           // block-Jacobi row blocks (1: global ILU)
    // element preconditioners (FG_PRECOND_LUE / SGSE): per element, in the
    // reference element order, its internal dofs (sink n) and 9 coefficients
    const int *ep_lmi;
    const double *ep_coef;
    // truncated SPIKE (precond == FG_PRECOND_SPIKE): sp_P row blocks of the
    // CSR operator, coupling size sp_k; band LU factors, k x k corner
    // couplings, LU of the 2k x 2k reduced systems; FP64 apply scratch
    int sp_k, sp_P, sp_smem_rows;
    const int *sp_bs, *sp_bl, *sp_bu;
    const long long *sp_boff;
    const double *sp_band, *sp_B, *sp_C, *sp_S;
    const int *sp_piv;
    double *sp_g, *sp_h, *sp_x;
    const double *A64;         // [S*S][nel_pad]
    const float *A32;
    const double *invd64;      // n_pad
    const float *invd32;
    const int *node_dof;       // [nnodes][ndof]
    const double *ibd64;       // [nnodes][ndof*ndof]
    const float *ibd32;
    double *x, *b, *ftrue, *r64, *t64, *u64;  // FP64 vectors (n_pad)
    void *V;                   // kmax vectors of T, stride n_pad
    void *w, *t;               // T vectors
    double *H;                 // (kmax+1) x kmax, H[j*kmax + i]
    double *g, *cs, *sn, *hbuf, *y;  // kmax+1 each
    double *G;                 // kmax x kmax Gram matrix of the basis (mixed precision)
    double *part;              // nparts x kPartStride
    unsigned *counter;         // 4 counters (one per reduction kernel kind)
    SysState *st;
};
constexpr int kIluWsChunk = 8;      // rows per staged chunk of the warp-per-block ILU substitutions
constexpr int kPartStride = 64;    // doubles per part (>= kmax + 2, kmax <= 60)

// Preconditioners applied by kernels of their own between the matvec and
// the Arnoldi pass (the others are fused into the vector kernels).
__host__ __device__ constexpr bool precond_separate(int p) { return p >= 2; }

struct EChunk { int sys, e0, e1; };
// One 3x3 patch of a batched matvec launch for the bulk-copy pipeline:
// system, first element, index-blob offset (16-byte units) and size
// (bytes), x segment start, and packed counts (elements | dofs << 16,
// incidence entries | x segment length << 16).
struct alignas(32) MvRec { int sys, pe0, boff16, bsize, xlo, pn, nx, pad; };
struct DChunk { int sys, part, d0, d1; };
struct NChunk { int sys, n0, n1; };

}  // namespace fg
