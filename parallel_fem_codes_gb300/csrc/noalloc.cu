// fg_matvec_noalloc: the EBE matvec of an existing system, with every piece
// of scratch memory it needs taken from one fixed array compiled into the
// library instead of from cudaMalloc.
//
// Who needs it: a host program whose device memory belongs to another
// allocator (a memory pool owned by a larger framework, or a solver loop
// that must not pay the implicit device synchronisation of cudaMalloc and
// cudaFree after its set-up phase).  Such a caller creates its systems once,
// during set-up, and afterwards can still run matvecs on device vectors it
// owns without the library allocating anything.
//
// Scratch.  g_noalloc_scratch is a file-scope __device__ array of
// kNoAllocBytes (about 33 MiB).  Every GPU that loads this library holds it
// until the process exits.  It stores the system descriptor, the matvec
// work-item table and two renumbering vectors of at most kNoAllocMaxEq entries,
// so the entry point accepts systems with n + 1 <= kNoAllocMaxEq equations
// (including the Dirichlet sink), at most kNoAllocMaxChunks element patches
// (a patch holds up to 1024 elements for 3x3 blocks, 256 for larger blocks)
// and at most kMaxColours patch colours, and rejects larger ones with
// FG_ERR_ARG.  It always multiplies by the element blocks (the EBE
// operator), also for a system switched to the assembled CSR operator
// (fg_set_operator), whose fg_matvec sums the same products in another
// order.  The host-side work-item table is one static array guarded by the
// same lock as the address table (the library allocates no host memory in
// this call either).
//
// Host code cannot use the array's name as a device address (in host code
// it names a host-side stand-in): the device address is looked up once per
// device with cudaGetSymbolAddress, with that device current, on the first
// call made on that device.  That first call should therefore come before
// any stream capture is started on the calling thread.
//
// Every call shares the one array and it keeps the last call's contents;
// the call clears what must start at zero.  Calls that overlap on the GPU
// (on different streams, or from different host threads) race on the array
// and must be serialised by the caller.
#include <cstring>
#include <mutex>

#include "system.h"

namespace fg {

constexpr int kNoAllocMaxEq = 1 << 21;       // n + 1 <= 2,097,152
constexpr int kNoAllocMaxChunks = 1 << 16;   // element patches (matvec work items) per system
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffDesc = 0;
constexpr size_t kOffCounts = align256(sizeof(SysDev));
constexpr size_t kOffChunks = kOffCounts + align256(sizeof(int) * kMaxColours);
constexpr size_t kOffX = kOffChunks + align256(sizeof(EChunk) * (size_t)kNoAllocMaxChunks);
constexpr size_t kOffY = kOffX + sizeof(double) * (size_t)kNoAllocMaxEq;
constexpr size_t kNoAllocBytes = kOffY + sizeof(double) * (size_t)kNoAllocMaxEq;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned char *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `dev` (which must be current).
// (the caller holds g_scratch_mu)
int scratch_on(int dev, unsigned char **out)
{
    if (dev < 0 || dev >= kMaxDevices) { set_error("fg_matvec_noalloc: device index out of range"); return FG_ERR_ARG; }
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return FG_OK;
}

__global__ void k_na_gather(const int *__restrict__ perm, const double *__restrict__ src, double *__restrict__ dst, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
    if (i == n) dst[n] = 0.0;
}

__global__ void k_na_scatter(const int *__restrict__ perm, const double *__restrict__ src, double *__restrict__ dst, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[perm[i]] = src[i];
    if (i == n) dst[n] = 0.0;
}

// host-side work-item table of a call (guarded by g_scratch_mu, held until
// its copy to the device has been staged)
EChunk g_chunks[kNoAllocMaxChunks];

}  // namespace
}  // namespace fg

using namespace fg;

extern "C" int fg_matvec_noalloc(fg_system *s, const double *P_dev, double *Q_dev, int precision)
{
    if (!s || !P_dev || !Q_dev) { set_error("fg_matvec_noalloc: NULL argument"); return FG_ERR_ARG; }
    if (precision != 64 && precision != 32) { set_error("fg_matvec_noalloc: precision must be 64 or 32"); return FG_ERR_ARG; }
    if (!s->blocks_ok) { set_error("fg_matvec_noalloc: element blocks were not set"); return FG_ERR_STATE; }
    const Topology &t = s->topo;
    if (t.n + 1 > kNoAllocMaxEq) {
        set_error("fg_matvec_noalloc: system has " + std::to_string(t.n + 1) +
                  " equations (with the sink), the fixed scratch holds at most " + std::to_string(kNoAllocMaxEq));
        return FG_ERR_ARG;
    }
    int dev = -1;
    FG_CUDA(cudaGetDevice(&dev));
    if (dev != s->device) { set_error("fg_matvec_noalloc: the system's device is not the current device"); return FG_ERR_ARG; }

    // matvec work items (one per patch of elements, grouped by patch colour)
    int off[kMaxColours + 1] = {0};
    int counts[kMaxColours] = {0};
    int nch = 0;
    if (t.npatch > kNoAllocMaxChunks) {
        set_error("fg_matvec_noalloc: system has " + std::to_string(t.npatch) + " element patches, the fixed "
                  "scratch holds at most " + std::to_string(kNoAllocMaxChunks));
        return FG_ERR_ARG;
    }
    if (t.npcol > kMaxColours) {
        set_error("fg_matvec_noalloc: system has " + std::to_string(t.npcol) + " patch colours, at most " +
                  std::to_string(kMaxColours) + " are supported");
        return FG_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    for (int c = 0; c < t.npcol; ++c) {
        for (int q = t.pc_ptr[c]; q < t.pc_ptr[c + 1]; ++q) g_chunks[nch++] = {0, t.pc_list[q], 0};
        off[c + 1] = nch;
        counts[c] = off[c + 1] - off[c];
    }

    unsigned char *base = nullptr;
    int r = scratch_on(dev, &base);
    if (r) return r;
    SysDev D{};
    D.n = t.n; D.n_pad = s->n_pad; D.nel = t.nel; D.nel_pad = s->nel_pad; D.S = t.S;
    D.lm = s->lm.as<int>(); D.A64 = s->A64.as<double>(); D.A32 = s->A32.as<float>();
    set_patch_fields(D, s);
    SysDev *d_desc = reinterpret_cast<SysDev *>(base + kOffDesc);
    int *d_counts = reinterpret_cast<int *>(base + kOffCounts);
    EChunk *d_chunks = reinterpret_cast<EChunk *>(base + kOffChunks);
    double *d_x = reinterpret_cast<double *>(base + kOffX);
    double *d_y = reinterpret_cast<double *>(base + kOffY);
    cudaStream_t st = s->stream;
    FG_CUDA(cudaMemcpyAsync(d_desc, &D, sizeof(SysDev), cudaMemcpyHostToDevice, st));
    if (t.npcol) FG_CUDA(cudaMemcpyAsync(d_counts, counts, sizeof(int) * t.npcol, cudaMemcpyHostToDevice, st));
    // pageable source: staged before the call returns, while the lock is held
    if (nch) FG_CUDA(cudaMemcpyAsync(d_chunks, g_chunks, sizeof(EChunk) * nch, cudaMemcpyHostToDevice, st));
    // x (reference numbering) -> internal numbering; y starts at zero
    k_na_gather<<<(t.n + 256) / 256, 256, 0, st>>>(s->perm.as<int>(), P_dev, d_x, t.n);
    FG_CUDA(cudaGetLastError());
    FG_CUDA(cudaMemsetAsync(d_y, 0, sizeof(double) * (size_t)(t.n + 1), st));
    if ((r = launch_matvec_colours(t.S, precision, d_desc, d_chunks, d_counts, off, t.npcol, t.maxdof, d_x, d_y, st)))
        return r;
    k_na_scatter<<<(t.n + 256) / 256, 256, 0, st>>>(s->perm.as<int>(), d_y, Q_dev, t.n);
    FG_CUDA(cudaGetLastError());
    count_launches(2);
    return FG_OK;
}
