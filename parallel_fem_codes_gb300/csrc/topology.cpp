// Host-side set-up of a mesh for the device: Fill_LM, local reverse
// Cuthill-McKee numbering, greedy element colouring, incidence lists.
// Runs once per mesh; everything per-iteration runs on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "fg_internal.h"
#include "../../include/femgpu.h"

namespace fg {

// ---------------------------------------------------------------- RCM
// Reverse Cuthill-McKee as 00_CommonFiles/Reordering/symrcm.c computes it
// (the permutation is part of the connectivity contract, so the order of
// every choice matters):
//  * degrees of the symmetrised pattern (calc_degrees, symrcm.c:307-350);
//  * neighbours visited in ascending index order, the union of row i of the
//    pattern and of its transpose (symrcm.c:136-199);
//  * unvisited neighbours go through a binary min-heap keyed on degree alone
//    with strict comparisons (H_insert/H_remove_min/H_heapify_min,
//    symrcm.c:508-567) before entering the BFS queue;
//  * each component starts at the node returned by the repeated-BFS
//    pseudo-peripheral search from its lowest unvisited index
//    (find_starting_node, symrcm.c:352-483);
//  * the Cuthill-McKee order is reversed at the end (symrcm.c:232-236).
namespace {
struct Cand { int id, deg, dist; };

struct MinHeap {
    std::vector<Cand> h;
    void push(Cand v) {
        size_t i = h.size();
        h.push_back(v);
        while (i > 0) {
            size_t p = (i - 1) / 2;
            if (h[i].deg < h[p].deg) { std::swap(h[i], h[p]); i = p; } else break;
        }
    }
    Cand pop() {
        Cand top = h[0];
        h[0] = h.back();
        h.pop_back();
        size_t n = h.size(), j = 0;
        for (;;) {
            size_t l = 2 * j + 1, r = 2 * j + 2, m = j;
            if (l < n && h[l].deg < h[j].deg) m = l;
            if (r < n && h[r].deg < h[m].deg) m = r;
            if (m == j) break;
            std::swap(h[j], h[m]);
            j = m;
        }
        return top;
    }
};

struct Graph {
    int n;
    const int *IA, *JA;
    std::vector<int> IT, JT, D;
    // ascending distinct neighbours of i (row i of A merged with row i of A^T)
    template <class F> void for_neighbours(int i, F &&f) const {
        int j1 = IA[i], e1 = IA[i + 1], j2 = IT[i], e2 = IT[i + 1];
        while (j1 < e1 || j2 < e2) {
            int r;
            if (j1 == e1) r = JT[j2++];
            else if (j2 == e2) r = JA[j1++];
            else {
                int a = JA[j1], b = JT[j2];
                if (a <= b) { r = a; ++j1; if (a == b) ++j2; }
                else { r = b; ++j2; }
            }
            f(r);
        }
    }
};

int pseudo_peripheral(const Graph &g, int start, std::vector<int> &seen, std::vector<Cand> &Q)
{
    Cand x{start, g.D[start], 0};
    int max_dist = 0;
    std::fill(seen.begin(), seen.end(), 0);
    size_t qh = 0;
    Q.clear();
    Q.push_back(x);
    seen[start] = 1;
    for (;;) {
        while (qh < Q.size()) {
            Cand v = Q[qh++];
            if (v.dist > x.dist || (v.id != x.id && v.deg > x.deg)) x = v;
            g.for_neighbours(v.id, [&](int r) {
                if (!seen[r]) { Q.push_back({r, g.D[r], v.dist + 1}); seen[r] = 1; }
            });
        }
        if (max_dist < x.dist) {
            max_dist = x.dist;
            std::fill(seen.begin(), seen.end(), 0);
            seen[x.id] = 1;
            x.dist = 0;
            Q.clear();
            qh = 0;
            Q.push_back(x);
        } else break;
    }
    return x.id;
}
}  // namespace

void symrcm(int n, const int *IA, const int *JA, int *perm)
{
    Graph g{n, IA, JA, {}, {}, {}};
    int nnz = IA[n];
    g.IT.assign(n + 1, 0);
    g.JT.assign(std::max(nnz, 1), 0);
    for (int k = 0; k < nnz; ++k) g.IT[JA[k] + 1]++;
    for (int i = 0; i < n; ++i) g.IT[i + 1] += g.IT[i];
    {
        std::vector<int> w(g.IT.begin(), g.IT.end());
        for (int i = 0; i < n; ++i)
            for (int k = IA[i]; k < IA[i + 1]; ++k) g.JT[w[JA[k]]++] = i;
    }
    g.D.assign(n, 0);
    int max_deg = 0;
    for (int i = 0; i < n; ++i)
        for (int k = IA[i]; k < IA[i + 1]; ++k) {
            int r = JA[k];
            max_deg = std::max(max_deg, ++g.D[r]);
            if (r != i) {
                bool found = false;
                for (int l = IA[r]; l < IA[r + 1]; ++l) {
                    if (JA[l] == i) { found = true; break; }
                    if (JA[l] > i) break;
                }
                if (!found) max_deg = std::max(max_deg, ++g.D[i]);
            }
        }
    if (max_deg == 0) {
        for (int i = 0; i < n; ++i) perm[i] = i;
        return;
    }
    std::vector<int> visit(n, 0), seen(n, 0);
    std::vector<Cand> Q, Q2;
    Q.reserve(n);
    Q2.reserve(n);
    MinHeap heap;
    size_t qh = 0;
    int c = 0;
    while (c < n) {
        int i = 0;
        while (i < n && visit[i]) ++i;
        Cand root{pseudo_peripheral(g, i, seen, Q2), 0, 0};
        root.deg = g.D[root.id];
        visit[root.id] = 1;
        Q.push_back(root);
        while (qh < Q.size()) {
            Cand v = Q[qh++];
            perm[c++] = v.id;
            g.for_neighbours(v.id, [&](int r) {
                if (!visit[r]) { heap.push({r, g.D[r], v.dist + 1}); visit[r] = 1; }
            });
            while (!heap.h.empty()) Q.push_back(heap.pop());
        }
    }
    std::reverse(perm, perm + n);
}

// MATRIX_bandwidth (reordering.c:215-236); the right band is taken from the
// last row only, as the reference's stray ';' makes it.
int matrix_bandwidth(int n, const int *IA, const int *JA)
{
    int bl = 0, br = 0;
    for (int i = 0; i < n; ++i) {
        if (std::fabs(double(i - JA[IA[i]])) > bl) bl = i - JA[IA[i]];
        br = JA[IA[i + 1] - 1] - i;
    }
    return std::max(bl, br);
}

// ---------------------------------------------------------------- topology
int build_topology(Topology &t, int nnodes, int nel, int ndof, const int *ien,
                   const int *type, const int *invp, int neq, int reorder)
{
    if (nnodes <= 0 || nel < 0 || ndof < 1 || ndof > 4 || neq < 0 || !ien || !type || !invp) {
        set_error("fg_system_create: invalid mesh arguments");
        return FG_ERR_ARG;
    }
    const int S = 3 * ndof, n = neq;
    t.nnodes = nnodes; t.nel = nel; t.ndof = ndof; t.S = S; t.n = n;
    t.ien.assign(ien, ien + (size_t)nel * 3);
    t.type.assign(type, type + (size_t)nnodes * ndof);
    t.invp.assign(invp, invp + (size_t)nnodes * ndof);
    for (size_t k = 0; k < t.ien.size(); ++k)
        if (t.ien[k] < 0 || t.ien[k] >= nnodes) { set_error("ien entry out of range"); return FG_ERR_ARG; }
    for (size_t d = 0; d < t.type.size(); ++d)
        if (t.type[d] != 0 && (t.invp[d] < 0 || t.invp[d] >= n)) {
            set_error("invp of a free dof out of range"); return FG_ERR_ARG;
        }

    // Fill_LM (01_SS_.../Fill_LM.c:3-27; 03_Euler_.../Fill_LM.c:3-31)
    t.lm.resize((size_t)nel * S);
    for (int e = 0; e < nel; ++e)
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < ndof; ++k) {
                int d = t.ien[3 * e + v] * ndof + k;
                t.lm[(size_t)e * S + ndof * v + k] = t.type[d] == 0 ? n : t.invp[d];
            }

    // dof adjacency (row-sorted, duplicate-free), Permutation_of_LM.c:21-49
    std::vector<int> IA(n + 1, 0), JA;
    {
        std::vector<int> cnt(n + 1, 0);
        for (int e = 0; e < nel; ++e)
            for (int a = 0; a < S; ++a) {
                int ra = t.lm[(size_t)e * S + a];
                if (ra == n) continue;
                for (int b = 0; b < S; ++b)
                    if (t.lm[(size_t)e * S + b] != n) cnt[ra]++;
            }
        std::vector<int> start(n + 1, 0);
        for (int r = 0; r < n; ++r) start[r + 1] = start[r] + cnt[r];
        std::vector<int> tmp(std::max(start[n], 1));
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int e = 0; e < nel; ++e)
            for (int a = 0; a < S; ++a) {
                int ra = t.lm[(size_t)e * S + a];
                if (ra == n) continue;
                for (int b = 0; b < S; ++b) {
                    int rb = t.lm[(size_t)e * S + b];
                    if (rb != n) tmp[start[ra] + cnt[ra]++] = rb;
                }
            }
        JA.reserve(start[n]);
        for (int r = 0; r < n; ++r) {
            std::sort(tmp.begin() + start[r], tmp.begin() + start[r + 1]);
            IA[r] = (int)JA.size();
            for (int k = start[r]; k < start[r + 1]; ++k)
                if (k == start[r] || tmp[k] != tmp[k - 1]) JA.push_back(tmp[k]);
        }
        IA[n] = (int)JA.size();
    }
    t.nnz = IA[n];
    t.perm.resize(n + 1);
    t.iperm.resize(n + 1);
    t.band_before = n > 0 ? matrix_bandwidth(n, IA.data(), JA.data()) : 0;
    if (reorder == FG_REORDER_RCM && n > 0) symrcm(n, IA.data(), JA.data(), t.perm.data());
    else std::iota(t.perm.begin(), t.perm.begin() + n, 0);
    t.perm[n] = n;
    for (int i = 0; i < n; ++i) t.iperm[t.perm[i]] = i;
    t.iperm[n] = n;
    t.band_after = t.band_before;
    if (n > 0 && reorder == FG_REORDER_RCM) {
        std::vector<int> IB(n + 1, 0), JB(t.nnz);
        for (int i = 0; i < n; ++i) IB[i + 1] = IB[i] + IA[t.perm[i] + 1] - IA[t.perm[i]];
        for (int i = 0; i < n; ++i) {
            int o = IB[i];
            for (int k = IA[t.perm[i]]; k < IA[t.perm[i] + 1]; ++k) JB[o++] = t.iperm[JA[k]];
            std::sort(JB.begin() + IB[i], JB.begin() + IB[i + 1]);
        }
        t.band_after = matrix_bandwidth(n, IB.data(), JB.data());
    }

    // greedy element colouring over the free dofs, in reference element order:
    // the smallest colour no earlier element sharing a free dof holds
    t.colour.assign(nel, 0);
    std::vector<uint64_t> used(n + 1, 0);
    std::vector<char> has_free(nel, 0);
    t.ncol = 0;
    for (int e = 0; e < nel; ++e) {
        uint64_t forb = 0;
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r != n) { forb |= used[r]; has_free[e] = 1; }
        }
        if (!has_free[e]) { t.colour[e] = -1; continue; }
        if (forb == ~0ull) { set_error("element colouring needs more than 64 colours"); return FG_ERR_UNSUPPORTED; }
        int c = __builtin_ctzll(~forb);
        t.colour[e] = c;
        t.ncol = std::max(t.ncol, c + 1);
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r != n) used[r] |= 1ull << c;
        }
    }
    // internal element order (the patch layout of the matvec): elements with
    // a free dof sorted by their smallest internal dof (stable), cut into
    // patches of patch_elems(S) consecutive elements; inside each patch the
    // elements are grouped by a greedy local colouring so that the patch's
    // shared-memory accumulation needs no atomics.  Elements without a free
    // dof go last and are skipped by the matvec.
    std::vector<int> key(nel);
    for (int e = 0; e < nel; ++e) {
        int m = n;
        for (int a = 0; a < S; ++a) m = std::min(m, t.iperm[t.lm[(size_t)e * S + a]]);
        key[e] = m;
    }
    std::vector<int> sorted(nel);
    std::iota(sorted.begin(), sorted.end(), 0);
    std::stable_sort(sorted.begin(), sorted.end(), [&](int a, int b) {
        int ka = has_free[a] ? key[a] : n + 1, kb = has_free[b] ? key[b] : n + 1;
        return ka < kb;
    });
    int nact = 0;
    for (int e = 0; e < nel; ++e) nact += has_free[e] ? 1 : 0;
    t.nel_active = nact;
    // A patch takes up to PE elements; it closes early, only at a multiple of
    // 16 elements (every patch starts 16-element aligned: aligned vector
    // loads of its rows), when 16 more elements could push its dof count
    // past the cap that bounds the matvec's shared memory.
    const int PE = patch_elems(S), dof_cap = S == 3 ? 1536 : PE * S;
    t.eorder.resize(nel);
    t.pt_elem.clear();
    t.pt_dof.clear();
    t.pt_xlo.clear();
    t.pt_xlen.clear();
    t.pt_col.clear();
    t.dofs.clear();
    t.maxdof = 0;
    std::vector<int> local(n + 1, -1), owner_count(n + 1, 0);
    std::vector<uint32_t> lmask;   // per local dof: local colours used
    for (int b = 0, p = 0; b < nact; ++p) {
        // local dofs of the patch, ascending internal index; a 3x3 patch also
        // keeps its dofs inside one x segment of at most kPatchXCap entries
        // (8-aligned ends): past that it goes back to its last 16-element
        // boundary
        std::vector<int> pd;
        int e = b, lo = n, hi = -1;
        size_t keep_pd = 0;
        int keep_lo = n, keep_hi = -1;
        while (e < nact && e - b < PE) {
            if ((e - b) % 16 == 0) {
                if ((int)pd.size() + 16 * S > dof_cap) break;
                keep_pd = pd.size(); keep_lo = lo; keep_hi = hi;
            }
            for (int a = 0; a < S; ++a) {
                int r = t.lm[(size_t)sorted[e] * S + a];
                if (r != n && local[t.iperm[r]] < 0) {
                    local[t.iperm[r]] = 0;
                    pd.push_back(t.iperm[r]);
                    lo = std::min(lo, t.iperm[r]);
                    hi = std::max(hi, t.iperm[r]);
                }
            }
            ++e;
            if (S == 3 && ((hi + 1 + 7) & ~7) - (lo & ~7) > kPatchXCap) {
                if (keep_pd == 0) { set_error("a 16-element group spans more than the matvec's x segment"); return FG_ERR_UNSUPPORTED; }
                for (size_t k = keep_pd; k < pd.size(); ++k) local[pd[k]] = -1;
                pd.resize(keep_pd);
                lo = keep_lo; hi = keep_hi;
                e = b + (int)((e - 1 - b) / 16) * 16;
                break;
            }
        }
        t.pt_elem.push_back(b);
        t.pt_col.resize((size_t)(p + 1) * kPatchColStride, 0);
        t.pt_dof.push_back(0);
        std::sort(pd.begin(), pd.end());
        t.pt_xlo.push_back(pd.front() & ~7);
        t.pt_xlen.push_back(((pd.back() + 1 + 7) & ~7) - (pd.front() & ~7));
        for (size_t j = 0; j < pd.size(); ++j) { local[pd[j]] = (int)j; owner_count[pd[j]]++; }
        // greedy local colouring in patch order
        lmask.assign(pd.size(), 0u);
        std::vector<int> lcol(e - b);
        int ncl = 0;
        for (int q = b; q < e; ++q) {
            uint32_t forb = 0;
            for (int a = 0; a < S; ++a) {
                int r = t.lm[(size_t)sorted[q] * S + a];
                if (r != n) forb |= lmask[local[t.iperm[r]]];
            }
            if ((forb & 0xFFFFu) == 0xFFFFu) {
                set_error("patch colouring needs more than 16 local colours"); return FG_ERR_UNSUPPORTED;
            }
            int c = __builtin_ctz(~forb);
            lcol[q - b] = c;
            ncl = std::max(ncl, c + 1);
            for (int a = 0; a < S; ++a) {
                int r = t.lm[(size_t)sorted[q] * S + a];
                if (r != n) lmask[local[t.iperm[r]]] |= 1u << c;
            }
        }
        // elements of the patch grouped by local colour (stable)
        std::vector<int> idx(e - b);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return lcol[x] < lcol[y]; });
        unsigned short *pc = &t.pt_col[(size_t)p * kPatchColStride];
        for (int c = 0, k = 0; c <= kPatchMaxLocalColours; ++c) {
            while (k < (int)idx.size() && lcol[idx[k]] < c) ++k;
            pc[c] = (unsigned short)k;     // first element of local colour c
        }
        for (int k = 0; k < (int)idx.size(); ++k) t.eorder[b + k] = sorted[b + idx[k]];
        // each patch's dof list starts on a 16-byte boundary
        while (t.dofs.size() % 4) t.dofs.push_back(n);
        t.pt_dof[p] = (int)t.dofs.size();
        for (int d : pd) t.dofs.push_back(d);
        t.maxdof = std::max(t.maxdof, (int)pd.size());
        for (int d : pd) local[d] = -1;
        b = e;
    }
    t.npatch = (int)t.pt_elem.size();
    t.pt_elem.push_back(nact);
    while (t.dofs.size() % 4) t.dofs.push_back(n);
    t.pt_dof.push_back((int)t.dofs.size());
    for (int q = nact; q < nel; ++q) t.eorder[q] = sorted[q];
    for (auto &d : t.dofs)
        if (owner_count[d] > 1) d |= (int)0x80000000u;
    t.epos.resize(nel);
    for (int p = 0; p < nel; ++p) t.epos[t.eorder[p]] = p;
    // patch-local element maps (internal element order)
    t.lm16.assign((size_t)nel * S, 0xFFFF);
    t.lmx16.assign((size_t)nel * S, 0xFFFF);
    for (int p = 0; p < t.npatch; ++p) {
        const int b = t.pt_elem[p], e = t.pt_elem[p + 1];
        for (int j = t.pt_dof[p]; j < t.pt_dof[p + 1]; ++j) local[t.dofs[j] & 0x7fffffff] = j - t.pt_dof[p];
        for (int q = b; q < e; ++q)
            for (int a = 0; a < S; ++a) {
                int r = t.lm[(size_t)t.eorder[q] * S + a];
                t.lm16[(size_t)q * S + a] = r == n ? (unsigned short)0xFFFF : (unsigned short)local[t.iperm[r]];
                t.lmx16[(size_t)q * S + a] = r == n ? (unsigned short)0xFFFF : (unsigned short)(t.iperm[r] - t.pt_xlo[p]);
            }
        for (int j = t.pt_dof[p]; j < t.pt_dof[p + 1]; ++j) local[t.dofs[j] & 0x7fffffff] = -1;
    }
    // incidence lists of the patches (summation of the staged products by dof)
    {
        const int PEs = patch_elems(S);
        t.pt_inc.assign(t.npatch + 1, 0);
        t.incl.clear();
        std::vector<int> cnt;
        for (int p = 0; p < t.npatch; ++p) {
            const int b = t.pt_elem[p], e = t.pt_elem[p + 1], nd = t.pt_dof[p + 1] - t.pt_dof[p];
            // staged products are rows of the patch width (3x3: its element
            // count rounded up to 16, the row length of the blocked FP32
            // blocks)
            const int Wp = S == 3 ? (e - b + 15) / 16 * 16 : PEs;
            t.pt_inc[p] = (int)t.incl.size();
            cnt.assign(nd + 1, 0);
            for (int q = b; q < e; ++q)
                for (int a = 0; a < S; ++a) {
                    const unsigned short l = t.lm16[(size_t)q * S + a];
                    if (l != 0xFFFF) cnt[l + 1]++;
                }
            for (int j = 0; j < nd; ++j) cnt[j + 1] += cnt[j];
            const size_t base = t.incl.size(), head = ((size_t)nd + 1 + 7) / 8 * 8;
            const size_t body = ((size_t)cnt[nd] + 7) / 8 * 8;
            t.incl.resize(base + head + body, 0);
            for (int j = 0; j <= nd; ++j) t.incl[base + j] = (unsigned short)cnt[j];
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            for (int q = b; q < e; ++q)
                for (int a = 0; a < S; ++a) {
                    const unsigned short l = t.lm16[(size_t)q * S + a];
                    if (l != 0xFFFF) t.incl[base + head + fill[l]++] = (unsigned short)(a * Wp + (q - b));
                }
        }
        t.pt_inc[t.npatch] = (int)t.incl.size();
    }
    // 3x3: one index blob per patch for the bulk-copy matvec, 16-byte
    // aligned: x-segment positions [3][W] (W = element count rounded up to
    // 16, padding 0xFFFF), the dof list, the incidence lists
    if (S == 3) {
        t.pt_boff.assign(t.npatch + 1, 0);
        t.blob.clear();
        for (int p = 0; p < t.npatch; ++p) {
            const int b = t.pt_elem[p], e = t.pt_elem[p + 1], W = (e - b + 15) / 16 * 16;
            t.pt_boff[p] = (long long)t.blob.size();
            const size_t o = t.blob.size();
            const size_t nd = t.pt_dof[p + 1] - t.pt_dof[p], ni = t.pt_inc[p + 1] - t.pt_inc[p];
            t.blob.resize(o + 6 * (size_t)W + 4 * nd + 2 * ni);
            unsigned short *lx = reinterpret_cast<unsigned short *>(t.blob.data() + o);
            for (int a = 0; a < 3; ++a)
                for (int i = 0; i < W; ++i) lx[a * W + i] = b + i < e ? t.lmx16[(size_t)(b + i) * 3 + a] : 0xFFFF;
            std::memcpy(t.blob.data() + o + 6 * (size_t)W, t.dofs.data() + t.pt_dof[p], 4 * nd);
            std::memcpy(t.blob.data() + o + 6 * (size_t)W + 4 * nd, t.incl.data() + t.pt_inc[p], 2 * ni);
        }
        t.pt_boff[t.npatch] = (long long)t.blob.size();
    }
    // patch colouring: patches that share a dof get different colours
    {
        std::vector<uint32_t> used(n + 1, 0u);
        std::vector<int> pcol(t.npatch, 0);
        t.npcol = 0;
        for (int p = 0; p < t.npatch; ++p) {
            uint32_t forb = 0;
            for (int j = t.pt_dof[p]; j < t.pt_dof[p + 1]; ++j)
                if (t.dofs[j] < 0) forb |= used[t.dofs[j] & 0x7fffffff];
            if (forb == 0xFFFFFFFFu) { set_error("patch colouring needs more than 32 colours"); return FG_ERR_UNSUPPORTED; }
            int c = __builtin_ctz(~forb);
            pcol[p] = c;
            t.npcol = std::max(t.npcol, c + 1);
            for (int j = t.pt_dof[p]; j < t.pt_dof[p + 1]; ++j)
                if (t.dofs[j] < 0) used[t.dofs[j] & 0x7fffffff] |= 1u << c;
        }
        t.pc_ptr.assign(t.npcol + 1, 0);
        for (int p = 0; p < t.npatch; ++p) t.pc_ptr[pcol[p] + 1]++;
        for (int c = 0; c < t.npcol; ++c) t.pc_ptr[c + 1] += t.pc_ptr[c];
        t.pc_list.assign(t.npatch, 0);
        std::vector<int> fill(t.pc_ptr.begin(), t.pc_ptr.end() - 1);
        for (int p = 0; p < t.npatch; ++p) t.pc_list[fill[pcol[p]]++] = p;
    }
    t.cptr.assign(t.ncol + 1, 0);

    // dof incidence: (pos, local row) per internal dof, reference element order
    t.dinc_ptr.assign(n + 1, 0);
    for (int e = 0; e < nel; ++e)
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r != n) t.dinc_ptr[t.iperm[r] + 1]++;
        }
    for (int i = 0; i < n; ++i) t.dinc_ptr[i + 1] += t.dinc_ptr[i];
    t.dinc.resize(std::max(t.dinc_ptr[n], 1));
    {
        std::vector<int> fill(t.dinc_ptr.begin(), t.dinc_ptr.end() - 1);
        for (int e = 0; e < nel; ++e)
            for (int a = 0; a < S; ++a) {
                int r = t.lm[(size_t)e * S + a];
                if (r != n) t.dinc[fill[t.iperm[r]]++] = t.epos[e] * 16 + a;
            }
    }
    // node incidence (pos, vertex), reference element order
    t.ninc_ptr.assign(nnodes + 1, 0);
    for (int e = 0; e < nel; ++e)
        for (int v = 0; v < 3; ++v) t.ninc_ptr[t.ien[3 * e + v] + 1]++;
    for (int i = 0; i < nnodes; ++i) t.ninc_ptr[i + 1] += t.ninc_ptr[i];
    t.ninc.resize(std::max(t.ninc_ptr[nnodes], 1));
    {
        std::vector<int> fill(t.ninc_ptr.begin(), t.ninc_ptr.end() - 1);
        for (int e = 0; e < nel; ++e)
            for (int v = 0; v < 3; ++v) t.ninc[fill[t.ien[3 * e + v]]++] = t.epos[e] * 4 + v;
    }
    t.node_dof.resize((size_t)nnodes * ndof);
    for (size_t d = 0; d < t.node_dof.size(); ++d)
        t.node_dof[d] = t.type[d] == 0 ? n : t.iperm[t.invp[d]];
    // The matvec kernels copy a patch's rows in 16-byte units: every patch
    // starts 16 elements aligned, its dof list and incidence lists start and
    // end on 16-byte boundaries and fit the kernels' shared-memory caps.
    {
        const int PE = patch_elems(S), dcap = S == 3 ? 1536 : PE * S;
        const int icap = (dcap + 1 + 7) / 8 * 8 + S * PE;
        const int nel_pad = std::max(32, (nel + 31) / 32 * 32);
        for (int p = 0; p < t.npatch; ++p) {
            const int pe0 = t.pt_elem[p], pne = t.pt_elem[p + 1] - pe0;
            const int pd0 = t.pt_dof[p], pnd = t.pt_dof[p + 1] - pd0;
            const int i0 = S == 3 ? t.pt_inc[p] : 0, ni = S == 3 ? t.pt_inc[p + 1] - i0 : 0;
            if (pe0 % 16 || pne < 1 || pne > PE || pe0 + (pne + 15) / 16 * 16 > nel_pad || pd0 % 4 || pnd % 4 ||
                pnd < 1 || pnd > dcap || i0 % 8 || ni % 8 || ni > icap ||
                (S == 3 && (t.pt_xlo[p] % 8 || t.pt_xlen[p] % 8 || t.pt_xlen[p] < 8 || t.pt_xlen[p] > kPatchXCap ||
                            t.pt_xlo[p] + t.pt_xlen[p] > (n + 1 + 31) / 32 * 32 || t.pt_boff[p] % 16 ||
                            t.pt_boff[p + 1] - t.pt_boff[p] > 6LL * PE + 4LL * dcap + 2LL * icap ||
                            t.pt_boff[p + 1] / 16 > 0x7fffffffLL))) {
                set_error("internal: matvec patch layout out of its bounds");
                return FG_ERR_UNSUPPORTED;
            }
        }
    }
    return FG_OK;
}

}  // namespace fg

namespace fg {

// Assembled CSR form (csr_Initialization.c:5-434): pattern of the free dofs
// in the internal numbering (the reference renumbers its equations by the
// same RCM, csr_Initialization.c:408-463), rows sorted, the diagonal slot of
// each row, and for every slot the element contributions in reference
// element order (csr_assembly.c sums them in that order).
int build_csr(const Topology &t, CsrTopology &c)
{
    const int n = t.n, S = t.S;
    c.n = n;
    c.ia.assign(n + 1, 0);
    std::vector<std::vector<int>> rows(n);
    for (int e = 0; e < t.nel; ++e)
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r == n) continue;
            for (int b = 0; b < S; ++b) {
                int q = t.lm[(size_t)e * S + b];
                if (q != n) rows[t.iperm[r]].push_back(t.iperm[q]);
            }
        }
    for (int i = 0; i < n; ++i) {
        auto &v = rows[i];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        c.ia[i + 1] = c.ia[i] + (int)v.size();
    }
    c.nnz = c.ia[n];
    c.ja.resize(std::max(c.nnz, 1));
    c.diag.assign(n, -1);
    for (int i = 0; i < n; ++i) {
        std::copy(rows[i].begin(), rows[i].end(), c.ja.begin() + c.ia[i]);
        for (int k = c.ia[i]; k < c.ia[i + 1]; ++k)
            if (c.ja[k] == i) c.diag[i] = k;
        if (c.diag[i] < 0) { set_error("CSR row without a diagonal entry"); return FG_ERR_ARG; }
        std::vector<int>().swap(rows[i]);
    }
    auto slot = [&](int r, int q) {
        const int *b = c.ja.data() + c.ia[r], *e = c.ja.data() + c.ia[r + 1];
        return (int)(std::lower_bound(b, e, q) - c.ja.data());
    };
    c.inc_ptr.assign(c.nnz + 1, 0);
    for (int e = 0; e < t.nel; ++e)
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r == n) continue;
            for (int b = 0; b < S; ++b) {
                int q = t.lm[(size_t)e * S + b];
                if (q != n) c.inc_ptr[slot(t.iperm[r], t.iperm[q]) + 1]++;
            }
        }
    for (int k = 0; k < c.nnz; ++k) c.inc_ptr[k + 1] += c.inc_ptr[k];
    c.inc.resize(std::max(c.inc_ptr[c.nnz], 1));
    std::vector<int> fill(c.inc_ptr.begin(), c.inc_ptr.end() - 1);
    for (int e = 0; e < t.nel; ++e)
        for (int a = 0; a < S; ++a) {
            int r = t.lm[(size_t)e * S + a];
            if (r == n) continue;
            for (int b = 0; b < S; ++b) {
                int q = t.lm[(size_t)e * S + b];
                if (q != n) c.inc[fill[slot(t.iperm[r], t.iperm[q])]++] = t.epos[e] * 256 + a * 16 + b;
            }
        }
    return FG_OK;
}

}  // namespace fg
