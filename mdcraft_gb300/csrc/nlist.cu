// nlist.cu — linked-cell binning and Verlet-list build on the device.
//
// Restates VerletList::update / build_linked_cells / are_neibs
// (mdcraft/neibs/verlet-list.cxx:41-55, 306-400) and Grid::build /
// adjacent_cells (mdcraft/neibs/grid.cxx:43-207) as a device pipeline:
//   wrap + bounds -> grid parameters -> bin count (bricked Morton keys)
//   -> exclusive scan -> scatter -> per-bin sort by caller index
//   -> permutation of every per-atom field -> warp-per-cell list build.
// The list test is the reference's FP64 expression evaluated without FMA
// contraction; an FP32 estimate from cell-centred offsets decides the clear
// cases and sends candidates within 1e-5 (relative) of the radius, or any
// geometry where the estimate is not provably the reference's image, to the
// exact FP64 test. Neighbour sets are therefore identical to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mdg_host.h"
#include "nlist_dev.cuh"

namespace mdg {

// ---------------------------------------------------------------------------
// bounds + wrap (Domain::fit_in_period, domain.cxx:41-47; Grid::find_bounds,
// grid.cxx:209-243)
// ---------------------------------------------------------------------------

__global__ void k_wrap_bounds(int n, double* __restrict__ rx, double* __restrict__ ry,
                              double* __restrict__ rz, const double* __restrict__ rns,
                              DomainDev d, double* __restrict__ part) {
    __shared__ double sh[7][kBlock];
    double lo[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double hi[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    double mr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double v[3];
        wrap_one(d, rx, ry, rz, i, v);
        for (int a = 0; a < 3; ++a) {
            lo[a] = fmin(lo[a], v[a]);
            hi[a] = fmax(hi[a], v[a]);
        }
        double q = rns[i];
        mr = mr < q ? q : mr;
    }
    int t = threadIdx.x;
    sh[0][t] = lo[0]; sh[1][t] = lo[1]; sh[2][t] = lo[2];
    sh[3][t] = hi[0]; sh[4][t] = hi[1]; sh[5][t] = hi[2];
    sh[6][t] = mr;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (t < s) {
            for (int k = 0; k < 3; ++k) sh[k][t] = fmin(sh[k][t], sh[k][t + s]);
            for (int k = 3; k < 7; ++k) sh[k][t] = fmax(sh[k][t], sh[k][t + s]);
        }
        __syncthreads();
    }
    if (t < 7) part[blockIdx.x * 8 + t] = sh[t][0];
}


__global__ void k_grid_finalize(const double* __restrict__ part, int nparts, DomainDev d,
                                GridParams* __restrict__ out, long long bin_cap, DevStatus* st) {
    __shared__ double sh[7][kBlock];
    int t = threadIdx.x;
    double v[7] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308,
                   -1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308, 0.0};
    for (int b = t; b < nparts; b += blockDim.x) {
        for (int k = 0; k < 3; ++k) v[k] = fmin(v[k], part[b * 8 + k]);
        for (int k = 3; k < 7; ++k) v[k] = fmax(v[k], part[b * 8 + k]);
    }
    for (int k = 0; k < 7; ++k) sh[k][t] = v[k];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (t < s) {
            for (int k = 0; k < 3; ++k) sh[k][t] = fmin(sh[k][t], sh[k][t + s]);
            for (int k = 3; k < 7; ++k) sh[k][t] = fmax(sh[k][t], sh[k][t + s]);
        }
        __syncthreads();
    }
    if (t != 0) return;
    GridParams g;
    double lo[3] = {sh[0][0], sh[1][0], sh[2][0]}, hi[3] = {sh[3][0], sh[4][0], sh[5][0]};
    grid_from_bounds(d, lo, hi, sh[6][0], g);
    if (g.empty == -1) {
        *out = g;
        return;
    }
    long long nb = g.nbins;
    // the bin arrays were sized on the host; a grid that outgrew them
    // invalidates this rebuild (every later kernel of it returns early)
    if (g.empty == 0 && nb + 1 > bin_cap) {
        g.empty = -3;
        atomicOr(&st->flags, FLAG_OVERFLOW);
        atomicOr(&st->build_flags, FLAG_OVERFLOW);
    }
    *out = g;
}

// ---------------------------------------------------------------------------
// binning: Grid::local_index3D + cell_index (grid.cxx:107-136) -> bin keys
// ---------------------------------------------------------------------------

__global__ void k_bin_count(int n, const double* __restrict__ rx, const double* __restrict__ ry,
                            const double* __restrict__ rz, const GridParams* __restrict__ gp,
                            uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                            uint32_t* __restrict__ bin_count, DevStatus* st) {
    const GridParams g = *gp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || g.empty) return;
    bin_count_one(g, i, rx, ry, rz, key, rank, bin_count, st);
}

// Exclusive scan of nb uint32 counts into start[0..nb] (start[nb] = total),
// 4096 items per block: per-block totals, a one-block scan of the totals,
// then per-block scans with offsets.
constexpr int kScanT = 1024, kScanItems = 4;


// Number of bins of the current rebuild (0 when the grid is invalid).
__device__ __forceinline__ int live_bins(const GridParams* gp) { return gp->empty ? 0 : gp->nbins; }

__global__ void k_scan_partial(const uint32_t* __restrict__ in, const GridParams* __restrict__ gp,
                               uint32_t* __restrict__ bsum) {
    __shared__ uint32_t sh[32];
    const int nb = live_bins(gp);
    int base = blockIdx.x * kScanT * kScanItems + threadIdx.x * kScanItems;
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) s += (base + k < nb) ? in[base + k] : 0u;
    uint32_t tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_top(uint32_t* __restrict__ bsum, const GridParams* __restrict__ gp) {
    __shared__ uint32_t sh[32];
    // block totals up to and including the block that holds index nb, whose
    // exclusive prefix is the grand total written to start[nb]
    const int nblk = live_bins(gp) / (kScanT * kScanItems) + 1;
    int base = threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < nblk) ? bsum[base + k] : 0u;
        s += v[k];
    }
    uint32_t off = block_excl_scan(s, sh, nullptr);
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < nblk) bsum[base + k] = off;
        off += v[k];
    }
}

__global__ void k_scan_final(const uint32_t* __restrict__ in, const GridParams* __restrict__ gp,
                             const uint32_t* __restrict__ bsum, uint32_t* __restrict__ out) {
    __shared__ uint32_t sh[32];
    const int nb = live_bins(gp);
    // blocks beyond the live bins (the grid is sized for the capacity) idle
    if (blockIdx.x * kScanT * kScanItems > nb) return;
    const int last = nb / (kScanT * kScanItems);
    int base = blockIdx.x * kScanT * kScanItems + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < nb) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t off = block_excl_scan(s, sh, &tot) + bsum[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < nb) out[base + k] = off;
        off += v[k];
    }
    if ((int)blockIdx.x == last && threadIdx.x == blockDim.x - 1) out[nb] = off;
}

__global__ void k_scatter(int n, const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                          const uint32_t* __restrict__ start, uint32_t* __restrict__ src,
                          const GridParams* __restrict__ gp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !gp->empty) src[start[key[i]] + rank[i]] = (uint32_t)i;
}

// Deterministic order inside a bin: ascending caller index.
__global__ void k_bin_sort(const GridParams* __restrict__ gp, const uint32_t* __restrict__ start,
                           uint32_t* __restrict__ src, const uint32_t* __restrict__ orig) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= live_bins(gp)) return;
    bin_sort_one(b, start, src, orig);
}

// Permutation of the per-atom fields: dst[k] = src_field[src[k]].

template <int NF, typename T>
__global__ void k_gather(int n, const uint32_t* __restrict__ src, GatherSet<NF, T> gs,
                         const GridParams* __restrict__ gp) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || gp->empty) return;
    uint32_t s = src[k];
#pragma unroll
    for (int f = 0; f < NF; ++f) gs.out[f][k] = gs.in[f][s];
}

// The permuted fields back into the live buffers (so device pointers stay
// fixed across rebuilds, as a captured graph needs).
template <int NF, typename T>
__global__ void k_copy(int n, GatherSet<NF, T> gs, const GridParams* __restrict__ gp) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || gp->empty) return;
#pragma unroll
    for (int f = 0; f < NF; ++f) gs.out[f][k] = gs.in[f][k];
}

// Cell centre, cell-relative FP32 offsets and packed cell of every atom.
__global__ void k_cells(int n, const double* __restrict__ rx, const double* __restrict__ ry,
                        const double* __restrict__ rz, const GridParams* __restrict__ gp,
                        uint32_t* __restrict__ cellp, double* __restrict__ Rx, double* __restrict__ Ry,
                        double* __restrict__ Rz, int4* __restrict__ pos32, int4* __restrict__ q0, float4* __restrict__ o0,
                        const uint32_t* __restrict__ orig, uint32_t* __restrict__ slot_of,
                        const uint16_t* __restrict__ kind) {
    const GridParams g = *gp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || g.empty) return;
    cells_one(g, i, rx, ry, rz, cellp, Rx, Ry, Rz, pos32, q0, o0, orig, slot_of, kind);
}

// ---------------------------------------------------------------------------
// VerletList::sort (verlet-list.cxx:237-249): atoms by Grid::cell_index
// (grid.cxx:134-136), x fastest. After a rebuild each cell's atoms are one
// run of slots (bricked keys) in ascending caller order, so an atom's place
// is its cell's start in x-fastest order plus its rank inside its bin.
// ---------------------------------------------------------------------------

__global__ void k_sort_cell_counts(const GridParams* __restrict__ gp, const uint32_t* __restrict__ bin_start,
                                   uint32_t* __restrict__ cnt, long long cap) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cap) return;
    const GridParams& g = *gp;
    if (g.empty || c >= (long long)g.num[0] * g.num[1] * g.num[2]) {
        cnt[c] = 0u;
        return;
    }
    const int cx = (int)(c % g.num[0]), cy = (int)((c / g.num[0]) % g.num[1]);
    const int cz = (int)(c / ((long long)g.num[0] * g.num[1]));
    const int b = bin_key(g, cx, cy, cz);
    cnt[c] = bin_start[b + 1] - bin_start[b];
}

__global__ void k_sort_place(int n, const GridParams* __restrict__ gp, const uint32_t* __restrict__ cellp,
                             const uint32_t* __restrict__ bin_start, const uint32_t* __restrict__ cell_start,
                             const uint32_t* __restrict__ orig, uint32_t* __restrict__ perm) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || gp->empty) return;
    const GridParams& g = *gp;
    int cx, cy, cz;
    unpack_cell(cellp[k], cx, cy, cz);
    const int b = bin_key(g, cx, cy, cz);
    const int c = cx + g.num[0] * (cy + g.num[1] * cz);
    perm[cell_start[c] + ((uint32_t)k - bin_start[b])] = orig[k];
}

// ---------------------------------------------------------------------------
// VerletList::list_for (verlet-list.cxx:251-276): the listed atoms of the
// query's adjacent cells within max(cell size, rns_j), a block per cell
// ---------------------------------------------------------------------------

struct ListForArgs {
    double x[3];
    double rad;
    bool edge[3];
    int bins[27];
};

__global__ void k_list_for(ListForArgs q, const GridParams* __restrict__ gp, const uint32_t* __restrict__ bin_start,
                           const double* __restrict__ rx, const double* __restrict__ ry,
                           const double* __restrict__ rz, const double* __restrict__ rns,
                           const uint32_t* __restrict__ orig, uint32_t* __restrict__ out,
                           uint32_t* __restrict__ count) {
    const GridParams& g = *gp;
    const int b = q.bins[blockIdx.x];
    for (uint32_t j = bin_start[b] + threadIdx.x; j < bin_start[b + 1]; j += blockDim.x) {
        if (are_neibs_exact(g, q.x[0], q.x[1], q.x[2], q.rad, rx[j], ry[j], rz[j], rns[j], q.edge))
            out[atomicAdd(count, 1u)] = orig[j];
    }
}

// ---------------------------------------------------------------------------
// VerletList::get() as CSR in caller order: per atom the atom itself and its
// stored entries (self padding dropped) as caller indices, ascending
// ---------------------------------------------------------------------------

__global__ void k_export_counts(int n, const uint32_t* __restrict__ slot_of, const uint32_t* __restrict__ ncnt,
                                const uint32_t* __restrict__ nbr, size_t np, uint32_t* __restrict__ cnt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const uint32_t s = slot_of[c];
    uint32_t m = 1;
    for (uint32_t k = 0; k < ncnt[s]; ++k) m += (nbr[nidx((int)k, s, np)] & kJMask) != s;
    cnt[c] = m;
}

// A warp per atom: the entries are collected in shared memory in list order,
// then each lane writes its entries at their ranks (the values are distinct:
// every neighbour appears once, the atom itself once). Lists longer than
// kExportWarpMax entries take a serial insertion on lane 0.
constexpr int kExportWarps = 8, kExportWarpMax = 256;

__global__ void __launch_bounds__(kExportWarps * 32)
    k_export_fill(int n, const uint32_t* __restrict__ slot_of, const uint32_t* __restrict__ ncnt,
                  const uint32_t* __restrict__ nbr, size_t np, const uint32_t* __restrict__ orig,
                  const uint64_t* __restrict__ off, uint64_t* __restrict__ idx) {
    __shared__ uint32_t buf[kExportWarps][kExportWarpMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * kExportWarps + w;
    if (c >= n) return;  // the whole warp
    const uint32_t s = slot_of[c], cnt = ncnt[s];
    uint64_t* seg = idx + off[c];
    const uint32_t len = (uint32_t)(off[c + 1] - off[c]);
    if (len > (uint32_t)kExportWarpMax) {
        if (lane != 0) return;
        seg[0] = (uint64_t)c;
        uint32_t m = 1;
        for (uint32_t k = 0; k < cnt && m < len; ++k) {
            const uint32_t j = nbr[nidx((int)k, s, np)] & kJMask;
            if (j == s) continue;
            const uint64_t v = orig[j];
            uint32_t p = m++;
            while (p > 0 && seg[p - 1] > v) {
                seg[p] = seg[p - 1];
                --p;
            }
            seg[p] = v;
        }
        return;
    }
    uint32_t* b = buf[w];
    if (lane == 0) b[0] = (uint32_t)c;
    uint32_t base = 1;
    for (uint32_t k0 = 0; k0 < cnt; k0 += 32) {
        const uint32_t k = k0 + lane;
        const uint32_t j = k < cnt ? (nbr[nidx((int)k, s, np)] & kJMask) : s;
        const bool keep = k < cnt && j != s;
        const unsigned mask = __ballot_sync(0xffffffffu, keep);
        const uint32_t pos = base + __popc(mask & ((1u << lane) - 1u));
        if (keep && pos < len) b[pos] = orig[j];
        base += __popc(mask);
    }
    __syncwarp();
    for (uint32_t p = lane; p < len; p += 32) {
        const uint32_t v = b[p];
        uint32_t r = 0;
        for (uint32_t q = 0; q < len; ++q) r += b[q] < v;
        seg[r] = v;
    }
}

// ---------------------------------------------------------------------------
// Verlet list
// ---------------------------------------------------------------------------

// Block of NW warps (cells per block: a system's launch shape, default 4),
// a warp per bin, on grids without a periodic axis of 2 cells or fewer
// (GridParams::small_box; those take k_nbuild_atoms). 64 registers.
template <int NW>
__global__ void __launch_bounds__(NW * 32, 32 / NW) k_nbuild_warp(NbArgs A, const GridParams* __restrict__ gp) {
    __shared__ GridParams g;
    __shared__ NbWarpSmem S[NW];
    if (threadIdx.x == 0) g = *gp;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bin = blockIdx.x * NW + warp;
    if (g.empty || g.small_box || bin >= g.nbins) return;
    nbuild_cell_warp(A, g, bin, lane, A.st->nonuniform == 0, S[warp]);
}

// The list build of grids with a periodic axis of 2 cells or fewer (a few
// cells of many atoms): a thread per atom. Launched after k_nbuild_warp. On
// the other grids it returns at once, unless some atom was clamped into the
// grid (FLAG_RANGE): those atoms' lists are built again from their
// unclamped cells (nbuild_atom), over what the warp build wrote.
__global__ void __launch_bounds__(kBlock) k_nbuild_atoms(NbArgs A, const GridParams* __restrict__ gp) {
    __shared__ GridParams g;
    if (threadIdx.x == 0) g = *gp;
    __syncthreads();
    if (g.empty) return;
    const bool clamped_only = !g.small_box;
    if (clamped_only && !(A.st->build_flags & FLAG_RANGE)) return;
    const bool uniform = A.st->nonuniform == 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (uint32_t)A.n; i += gridDim.x * blockDim.x)
        if (!clamped_only || A.o0[i].w == 2.0f) nbuild_atom(A, g, i, uniform);
}

// VerletList::optimize_search_radius (verlet-list.cxx:72-92):
// rns_i = kbuf * max over the current list of (rcut_i + rcut_j).
__global__ void k_optimize_rns(int n, int np, double kbuf, int have_list, const uint32_t* __restrict__ nbr,
                               const uint32_t* __restrict__ ncnt, const double* __restrict__ rcut,
                               double* __restrict__ rns) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double hmax = 0.0;
    if (have_list) {
        double ri = rcut[i];
        // the reference's list includes the atom itself
        hmax = ri + ri;
        int c = ncnt[i];
        for (int k = 0; k < c; ++k) {
            uint32_t j = nbr[nidx(k, i, np)] & kJMask;
            double h = ri + rcut[j];
            hmax = h > hmax ? h : hmax;
        }
    }
    rns[i] = kbuf * hmax;
}

__global__ void k_check_rns(int n, const double* __restrict__ rns, DevStatus* st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && rns[i] != rns[0]) atomicOr(&st->nonuniform, 1u);
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

static int ensure_bins(mdg_system* sys, long long nbins) {
    if ((size_t)nbins + 1 <= sys->bin_cap) return MDG_OK;
    size_t cap = (size_t)nbins + 1;
    cap = cap + cap / 8 + 4096;
    sys_free(sys, sys->bin_count, sys->bin_cap * sizeof(uint32_t));
    sys_free(sys, sys->bin_start, sys->bin_cap * sizeof(uint32_t));
    sys_free(sys, sys->scan_tmp, sys->scan_cap * sizeof(uint32_t));
    sys->bin_count = sys->bin_start = sys->scan_tmp = nullptr;
    sys->bin_cap = sys->scan_cap = 0;
    size_t scan = cap / (kScanT * kScanItems) + 2;
    int rc = sys_malloc(sys, (void**)&sys->bin_count, cap * sizeof(uint32_t));
    if (!rc) rc = sys_malloc(sys, (void**)&sys->bin_start, cap * sizeof(uint32_t));
    if (!rc) rc = sys_malloc(sys, (void**)&sys->scan_tmp, scan * sizeof(uint32_t));
    if (rc) return rc;
    sys->bin_cap = cap;
    sys->scan_cap = scan;
    sys->cap_version++;
    return MDG_OK;
}

static int ensure_list(mdg_system* sys, int K) {
    K = (K + 3) & ~3;
    if (K <= sys->K && sys->nbr) return MDG_OK;
    sys_free(sys, sys->nbr, (size_t)sys->K * sys->np * sizeof(uint32_t));
    sys->nbr = nullptr;
    sys->K = 0;
    int rc = sys_malloc(sys, (void**)&sys->nbr, (size_t)K * sys->np * sizeof(uint32_t));
    if (rc) return rc;
    sys->K = K;
    sys->cap_version++;
    return MDG_OK;
}

static DomainDev domain_dev(const mdg_system* sys) {
    DomainDev d;
    for (int a = 0; a < 3; ++a) {
        d.bmin[a] = sys->dom.bmin[a];
        d.bmax[a] = sys->dom.bmax[a];
        d.size[a] = sys->dom.bmax[a] - sys->dom.bmin[a];
        d.periodic[a] = sys->dom.periodic[a] ? 1 : 0;
    }
    d.dim = sys->dim;
    return d;
}

static int nparts_of(const mdg_system* sys) {
    return std::min(nblk(sys->n), 8 * std::max(sys->ctx->num_sms, 1));
}

static int ensure_parts(mdg_system* sys) {
    int nparts = nparts_of(sys);
    if ((size_t)nparts > sys->part_cap) {
        sys_free(sys, sys->part, sys->part_cap * 8 * sizeof(double));
        sys->part = nullptr;
        sys->part_cap = 0;
        int rc = sys_malloc(sys, (void**)&sys->part, (size_t)nparts * 8 * sizeof(double));
        if (rc) return rc;
        sys->part_cap = nparts;
    }
    return MDG_OK;
}

int size_from_grid(mdg_system* sys, const GridParams& g, int half);

// Sizes the bin arrays and the list capacity from one synchronous bounds
// pass (positions are wrapped by it exactly as by a rebuild).
int nlist_capacity(mdg_system* sys, int half) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)sys->n;
    int rc = ensure_parts(sys);
    if (rc) return rc;
    int nparts = nparts_of(sys);
    DomainDev d = domain_dev(sys);
    int c = sys->cur;
    k_wrap_bounds<<<nparts, kBlock, 0, st>>>(n, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c],
                                             sys->f64[RNS][c], d, sys->part);
    MDG_LAUNCHED(ctx);
    k_grid_finalize<<<1, kBlock, 0, st>>>(sys->part, nparts, d, sys->dgrid, 1LL << 40, sys->dstat);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(sys->hgrid, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    return size_from_grid(sys, *sys->hgrid, half);
}

// Grid::build alone: the bounds pass and the grid of the current positions.
int grid_build_only(mdg_system* sys, GridParams* out) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    int rc = ensure_parts(sys);
    if (rc) return rc;
    const int nparts = nparts_of(sys);
    DomainDev d = domain_dev(sys);
    const int c = sys->cur;
    k_wrap_bounds<<<nparts, kBlock, 0, st>>>((int)sys->n, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c],
                                             sys->f64[RNS][c], d, sys->part);
    MDG_LAUNCHED(ctx);
    k_grid_finalize<<<1, kBlock, 0, st>>>(sys->part, nparts, d, sys->dgrid, 1LL << 40, sys->dstat);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(out, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    if (out->empty == -1) {
        set_error("neighbour search radius rns must be positive");
        return MDG_ERR_INVALID;
    }
    if (out->empty == -2) {
        set_error("cell grid too large (more than 1023 cells on an axis)");
        return MDG_ERR_INVALID;
    }
    return MDG_OK;
}

// The same sizing from atoms still on the host (before they are uploaded):
// the bounds pass is repeated on the host with the device's arithmetic, so
// the grid is the one the first rebuild will compute. Nothing waits for the
// device.
int nlist_capacity_host(mdg_system* sys, const mdg_atom* atoms, size_t n, int half) {
    int rc = ensure_parts(sys);
    if (rc) return rc;
    DomainDev d = domain_dev(sys);
    double lo[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double hi[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    double mr = 0.0;
    for (size_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            double v = atoms[i].r[a];
            if (d.periodic[a]) v = v < d.bmin[a] ? v + d.size[a] : v > d.bmax[a] ? v - d.size[a] : v;
            lo[a] = std::min(lo[a], v);
            hi[a] = std::max(hi[a], v);
        }
        mr = std::max(mr, atoms[i].rns);
    }
    GridParams g;
    grid_from_bounds(d, lo, hi, mr, g);
    *sys->hgrid = g;
    return size_from_grid(sys, g, half);
}

// Bin arrays and list capacity for grid g (the grid of the next rebuild).
int size_from_grid(mdg_system* sys, const GridParams& g, int half) {
    const int n = (int)sys->n;
    int rc;
    if (g.empty == -1) {
        set_error("neighbour search radius rns must be positive");
        return MDG_ERR_INVALID;
    }
    if (g.empty == -2) {
        set_error("cell grid too large (more than 1023 cells on an axis)");
        return MDG_ERR_INVALID;
    }
    // periodic axes keep their grid; open axes get room to grow
    long long want = g.nbins;
    bool open = false;
    for (int a = 0; a < sys->dim; ++a) open = open || !sys->dom.periodic[a];
    if (open) want = want * 2;
    rc = ensure_bins(sys, want);
    if (rc) return rc;
    if (sys->K == 0 || sys->half != half) {
        double vol = 1.0;
        for (int a = 0; a < sys->dim; ++a) vol *= g.cs[a] * g.num[a];
        double dens = (double)n / std::max(vol, 1e-300);
        double rn = g.max_rns;
        // neighbours within rns at the mean density of the local grid (an open
        // system's grid also holds empty space: the retry grows K if needed)
        double est = sys->dim == 3 ? 4.18879020478639 * rn * rn * rn * dens
                   : sys->dim == 2 ? 3.14159265358979 * rn * rn * dens : 2.0 * rn * dens;
        if (open) est *= 2.0;
        if (half) est *= 0.5;
        int K = (int)(est * 1.35) + 16;
        K = std::min(std::max(K, 16), n + 4);
        rc = ensure_list(sys, K);
        if (rc) return rc;
    }
    sys->half = half;
    sys->cap_ready = 1;
    return MDG_OK;
}

// Enqueues a whole rebuild on the context stream with no host
// synchronisation: every size comes from the device grid parameters, and a
// grid or list that outgrows the capacities raises FLAG_OVERFLOW in
// build_flags (the kernels of an invalid grid return early).
GatherAll gather_sets(const mdg_system* sys) {
    const int c = sys->cur, alt = c ^ 1;
    GatherAll G;
    for (int f = 0; f < 12; ++f) {
        G.a.in[f] = sys->f64[f][c];
        G.a.out[f] = sys->f64[f][alt];
        G.b.in[f] = sys->f64[12 + f][c];
        G.b.out[f] = sys->f64[12 + f][alt];
        G.a2.in[f] = G.a.out[f];
        G.a2.out[f] = sys->f64[f][c];
        G.b2.in[f] = G.b.out[f];
        G.b2.out[f] = sys->f64[12 + f][c];
    }
    for (int f = 0; f < 3; ++f) {
        G.fc.in[f] = sys->f32[f][c];
        G.fc.out[f] = sys->f32[f][alt];
        G.fc2.in[f] = G.fc.out[f];
        G.fc2.out[f] = sys->f32[f][c];
    }
    for (int f = 0; f < 2; ++f) {
        G.u.in[f] = sys->u32[f][c];
        G.u.out[f] = sys->u32[f][alt];
        G.u2.in[f] = G.u.out[f];
        G.u2.out[f] = sys->u32[f][c];
        G.h.in[f] = sys->u16[f][c];
        G.h.out[f] = sys->u16[f][alt];
        G.h2.in[f] = G.h.out[f];
        G.h2.out[f] = sys->u16[f][c];
    }
    return G;
}

NbArgs nb_args(const mdg_system* sys) {
    const int c = sys->cur;
    NbArgs A;
    A.n = (int)sys->n;
    A.np = (int)sys->np;
    A.K = sys->K;
    A.half = sys->half;
    A.rx = sys->f64[RX][c];
    A.ry = sys->f64[RY][c];
    A.rz = sys->f64[RZ][c];
    A.rns = sys->f64[RNS][c];
    A.rcut = sys->f64[RCUT][c];
    A.orig = sys->u32[ORIG][c];
    A.uid = sys->u32[UID][c];
    A.cellp = sys->cellp;
    A.bin_start = sys->bin_start;
    A.o0 = sys->o0;
    A.nbr = sys->nbr;
    A.ncnt = sys->ncnt;
    A.r0x = sys->r0[0];
    A.r0y = sys->r0[1];
    A.r0z = sys->r0[2];
    A.saved_rcut = sys->saved_rcut;
    A.saved_rns = sys->saved_rns;
    A.saved_uid = sys->saved_uid;
    A.st = sys->dstat;
    return A;
}

DomainDev domain_of(const mdg_system* sys) { return domain_dev(sys); }

// Lanes per cell of the list build: 16, or 32 when the cells of the last
// sized grid hold more than 16 atoms on average.

int nlist_enqueue(mdg_system* sys) {
    mdg_ctx* ctx = sys->ctx;
    sys->fp_ok = 0;  // the atoms are permuted; Fp64 is per slot
    cudaStream_t st = ctx->stream;
    const int n = (int)sys->n;
    if (n == 0) return MDG_OK;
    int nparts = nparts_of(sys);
    DomainDev d = domain_dev(sys);
    const int c = sys->cur;
    MDG_CUDA(cudaMemsetAsync(&sys->dstat->max_count, 0, 3 * sizeof(uint32_t), st));  // max_count, nonuniform, build_flags
    k_wrap_bounds<<<nparts, kBlock, 0, st>>>(n, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c],
                                             sys->f64[RNS][c], d, sys->part);
    MDG_LAUNCHED(ctx);
    k_grid_finalize<<<1, kBlock, 0, st>>>(sys->part, nparts, d, sys->dgrid, (long long)sys->bin_cap, sys->dstat);
    MDG_LAUNCHED(ctx);
    k_check_rns<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RNS][c], sys->dstat);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemsetAsync(sys->bin_count, 0, sys->bin_cap * sizeof(uint32_t), st));
    k_bin_count<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c], sys->dgrid,
                                            sys->key, sys->rank, sys->bin_count, sys->dstat);
    MDG_LAUNCHED(ctx);
    int nscan = (int)((sys->bin_cap + kScanT * kScanItems - 1) / (kScanT * kScanItems));
    if (nscan > kScanT * kScanItems) {
        set_error("too many cell bins for the scan");
        return MDG_ERR_INVALID;
    }
    k_scan_partial<<<nscan, kScanT, 0, st>>>(sys->bin_count, sys->dgrid, sys->scan_tmp);
    MDG_LAUNCHED(ctx);
    k_scan_top<<<1, kScanT, 0, st>>>(sys->scan_tmp, sys->dgrid);
    MDG_LAUNCHED(ctx);
    k_scan_final<<<nscan, kScanT, 0, st>>>(sys->bin_count, sys->dgrid, sys->scan_tmp, sys->bin_start);
    MDG_LAUNCHED(ctx);
    k_scatter<<<nblk(n), kBlock, 0, st>>>(n, sys->key, sys->rank, sys->bin_start, sys->src, sys->dgrid);
    MDG_LAUNCHED(ctx);
    k_bin_sort<<<nblk(sys->bin_cap), kBlock, 0, st>>>(sys->dgrid, sys->bin_start, sys->src, sys->u32[ORIG][c]);
    MDG_LAUNCHED(ctx);
    // permute every per-atom field into the spare buffers, then copy back
    {
        GatherAll G = gather_sets(sys);
        auto& a = G.a; auto& b = G.b; auto& a2 = G.a2; auto& b2 = G.b2;
        auto& fc = G.fc; auto& fc2 = G.fc2; auto& u = G.u; auto& u2 = G.u2; auto& h = G.h; auto& h2 = G.h2;
        k_gather<12, double><<<nblk(n), kBlock, 0, st>>>(n, sys->src, a, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_gather<12, double><<<nblk(n), kBlock, 0, st>>>(n, sys->src, b, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_gather<3, float><<<nblk(n), kBlock, 0, st>>>(n, sys->src, fc, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_gather<2, uint32_t><<<nblk(n), kBlock, 0, st>>>(n, sys->src, u, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_gather<2, uint16_t><<<nblk(n), kBlock, 0, st>>>(n, sys->src, h, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_copy<12, double><<<nblk(n), kBlock, 0, st>>>(n, a2, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_copy<12, double><<<nblk(n), kBlock, 0, st>>>(n, b2, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_copy<3, float><<<nblk(n), kBlock, 0, st>>>(n, fc2, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_copy<2, uint32_t><<<nblk(n), kBlock, 0, st>>>(n, u2, sys->dgrid);
        MDG_LAUNCHED(ctx);
        k_copy<2, uint16_t><<<nblk(n), kBlock, 0, st>>>(n, h2, sys->dgrid);
        MDG_LAUNCHED(ctx);
    }
    k_cells<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c], sys->dgrid,
                                        sys->cellp, sys->Rc[0], sys->Rc[1], sys->Rc[2], sys->pos32, sys->q0, sys->o0,
                                        sys->u32[ORIG][c], sys->slot_of, sys->u16[KIND][c]);
    MDG_LAUNCHED(ctx);
    NbArgs A = nb_args(sys);
    // a half warp per bin of the capacity (a whole warp where cells hold more
    // than 16 atoms on average); the live bins come from the device grid
    const int cpb = sys->shape[MDG_SHAPE_LIST_CELLS_PER_BLOCK] ? sys->shape[MDG_SHAPE_LIST_CELLS_PER_BLOCK] : 4;
    const unsigned nbw = (unsigned)((sys->bin_cap + cpb - 1) / cpb);
    if (cpb == 2) k_nbuild_warp<2><<<nbw, 2 * 32, 0, st>>>(A, sys->dgrid);
    else if (cpb == 8) k_nbuild_warp<8><<<nbw, 8 * 32, 0, st>>>(A, sys->dgrid);
    else k_nbuild_warp<4><<<nbw, 4 * 32, 0, st>>>(A, sys->dgrid);
    MDG_LAUNCHED(ctx);
    // a grid-stride launch of at most four blocks per SM: on the large
    // grids, where it returns at once, its blocks are few
    k_nbuild_atoms<<<std::min(nblk(n), 4 * std::max(ctx->num_sms, 1)), kBlock, 0, st>>>(A, sys->dgrid);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

static int sort_perm_enqueue(mdg_system* sys, uint32_t* cell_start, uint32_t* perm) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)sys->n;
    const long long cap = (long long)sys->bin_cap;
    // the bin counts are free after the rebuild's scan: they take the
    // per-cell counts in x-fastest order, scanned like the bins
    k_sort_cell_counts<<<nblk((size_t)cap), kBlock, 0, st>>>(sys->dgrid, sys->bin_start, sys->bin_count, cap);
    MDG_LAUNCHED(ctx);
    const int nscan = (int)((cap + kScanT * kScanItems - 1) / (kScanT * kScanItems));
    k_scan_partial<<<nscan, kScanT, 0, st>>>(sys->bin_count, sys->dgrid, sys->scan_tmp);
    MDG_LAUNCHED(ctx);
    k_scan_top<<<1, kScanT, 0, st>>>(sys->scan_tmp, sys->dgrid);
    MDG_LAUNCHED(ctx);
    k_scan_final<<<nscan, kScanT, 0, st>>>(sys->bin_count, sys->dgrid, sys->scan_tmp, cell_start);
    MDG_LAUNCHED(ctx);
    k_sort_place<<<nblk(n), kBlock, 0, st>>>(n, sys->dgrid, sys->cellp, sys->bin_start, cell_start,
                                             sys->u32[ORIG][sys->cur], perm);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaStreamSynchronize(st));
    return MDG_OK;
}

// perm[p] = caller index of the atom at place p of VerletList::sort, from
// the grid and bins of the rebuild just done on `sys` (waits for it). The
// bin counts are overwritten; the list and the atoms are not touched.
int nlist_sort_perm(mdg_system* sys, uint32_t* perm) {
    if (sys->n == 0) return MDG_OK;
    if (!sys->have_list || sys->grid.empty) {
        set_error("no cell grid to sort by");
        return MDG_ERR_INVALID;
    }
    uint32_t* cell_start = nullptr;
    MDG_CUDA(cudaMalloc(&cell_start, ((size_t)sys->bin_cap + 1) * sizeof(uint32_t)));
    const int rc = sort_perm_enqueue(sys, cell_start, perm);
    cudaFree(cell_start);
    return rc;
}

// The caller indices list_for(x) finds, ascending (the reference's list in
// cell-walk order, as a set). The adjacent cells follow Grid::adjacent_cells
// (grid.cxx:138-207) on the grid of the last rebuild.
int nlist_list_for(mdg_system* sys, const double x[3], std::vector<uint64_t>& found) {
    found.clear();
    if (sys->n == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    // the grid of the last rebuild, which may have run inside a device loop
    GridParams g;
    MDG_CUDA(cudaMemcpyAsync(&g, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    if (g.empty) return MDG_OK;
    ListForArgs q;
    memset(&q, 0, sizeof(q));
    int cell[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a) q.x[a] = x[a];
    for (int a = 0; a < g.dim; ++a) cell[a] = (int)std::floor((x[a] - g.bmin[a]) / g.cs[a]);
    for (int a = 0; a < g.dim; ++a) q.edge[a] = cell[a] == 0 || cell[a] == g.num[a] - 1;
    q.rad = std::max(g.cs[0], std::max(g.cs[1], g.cs[2]));
    int nb = 0;
    for (int dx = -1; dx <= 1; ++dx) {
        if (g.periodic[0] && ((g.dom_n[0] == 1 && dx != 0) || (g.dom_n[0] == 2 && dx == 1))) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            if (g.periodic[1] && ((g.dom_n[1] == 1 && dy != 0) || (g.dom_n[1] == 2 && dy == 1))) continue;
            for (int dz = -1; dz <= 1; ++dz) {
                if (g.periodic[2] && ((g.dom_n[2] == 1 && dz != 0) || (g.dom_n[2] == 2 && dz == 1))) continue;
                int c[3] = {cell[0] + dx, cell[1] + dy, cell[2] + dz};
                for (int a = 0; a < 3; ++a)
                    if (g.periodic[a]) c[a] = (c[a] + g.dom_n[a]) % g.dom_n[a];
                int lc[3] = {c[0] - g.offset[0], c[1] - g.offset[1], c[2] - g.offset[2]};
                bool in = true;
                for (int a = 0; a < 3; ++a) in = in && lc[a] >= 0 && lc[a] < g.num[a];
                if (in) q.bins[nb++] = bin_key(g, lc[0], lc[1], lc[2]);
            }
        }
    }
    if (nb == 0) return MDG_OK;
    const int c = sys->cur;
    // results land in the spare slot-order buffers (free between rebuilds)
    uint32_t* out = sys->key;
    uint32_t* cnt = sys->rank;
    MDG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t), st));
    k_list_for<<<nb, 128, 0, st>>>(q, sys->dgrid, sys->bin_start, sys->f64[RX][c], sys->f64[RY][c],
                                   sys->f64[RZ][c], sys->f64[RNS][c], sys->u32[ORIG][c], out, cnt);
    MDG_LAUNCHED(ctx);
    uint32_t m = 0;
    MDG_CUDA(cudaMemcpyAsync(&m, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> idx(m);
    if (m) MDG_CUDA(cudaMemcpy(idx.data(), out, m * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    found.assign(idx.begin(), idx.end());
    std::sort(found.begin(), found.end());
    return MDG_OK;
}

// CSR offsets (n + 1) of the exported list, counted on the device.
int nlist_export_offsets(mdg_system* sys, std::vector<uint64_t>& off) {
    const size_t n = sys->n;
    off.assign(n + 1, 0);
    if (n == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    // the spare slot-order buffer takes the counts (free between rebuilds)
    uint32_t* cnt = sys->key;
    k_export_counts<<<nblk(n), kBlock, 0, st>>>((int)n, sys->slot_of, sys->ncnt, sys->nbr, sys->np, cnt);
    MDG_LAUNCHED(ctx);
    std::vector<uint32_t> h(n);
    MDG_CUDA(cudaMemcpyAsync(h.data(), cnt, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    for (size_t c = 0; c < n; ++c) off[c + 1] = off[c] + h[c];
    return MDG_OK;
}

// The exported entries (off[n] of them) into the host array idx.
int nlist_export_entries(mdg_system* sys, const std::vector<uint64_t>& off, uint64_t* idx) {
    const size_t n = sys->n, total = off[n];
    if (total == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    uint64_t *doff = nullptr, *didx = nullptr;
    MDG_CUDA(cudaMalloc(&doff, (n + 1) * sizeof(uint64_t)));
    if (cudaMalloc(&didx, total * sizeof(uint64_t)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(doff);
        set_error("no device memory for the list export");
        return MDG_ERR_NOMEM;
    }
    int rc = MDG_OK;
    cudaError_t e = cudaMemcpyAsync(doff, off.data(), (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_export_fill<<<(unsigned)((n + kExportWarps - 1) / kExportWarps), kExportWarps * 32, 0, st>>>(
            (int)n, sys->slot_of, sys->ncnt, sys->nbr, sys->np, sys->u32[ORIG][sys->cur], doff, didx);
        ctx->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx, didx, total * sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "list export");
    cudaFree(didx);
    cudaFree(doff);
    return rc;
}

int launch_trig(mdg_system* sys);

// VerletList::update (verlet-list.cxx:41-55) for the API: enqueue, wait,
// and rebuild again with larger capacities when the grid or a list outgrew
// them.
int nlist_build(mdg_system* sys, double kbuf, int half) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)sys->n;
    if (n == 0) {
        sys->have_list = 1;
        sys->half = half;
        sys->dirty = 0;
        return MDG_OK;
    }
    int c = sys->cur;
    if (kbuf > 0.0) {
        k_optimize_rns<<<nblk(n), kBlock, 0, st>>>(n, (int)sys->np, kbuf, sys->have_list, sys->nbr, sys->ncnt,
                                                   sys->f64[RCUT][c], sys->f64[RNS][c]);
        MDG_LAUNCHED(ctx);
        sys->cap_ready = 0;  // rns changed: re-size the grid
    }
    int rc;
    if (!sys->cap_ready || sys->half != half) {
        rc = nlist_capacity(sys, half);
        if (rc) return rc;
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        rc = nlist_enqueue(sys);
        if (rc) return rc;
        rc = launch_trig(sys);
        if (rc) return rc;
        MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
        MDG_CUDA(cudaMemcpyAsync(sys->hgrid, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, st));
        MDG_CUDA(cudaStreamSynchronize(st));
        if (!(sys->hstat->build_flags & FLAG_OVERFLOW)) break;
        // grow what overflowed and rebuild (the positions are already wrapped
        // and sorted, so a repeated rebuild gives the same order)
        GridParams g = *sys->hgrid;
        if (g.empty == -3) {
            rc = nlist_capacity(sys, half);
            if (rc) return rc;
        }
        if ((int)sys->hstat->max_count > sys->K) {
            rc = ensure_list(sys, (int)(sys->hstat->max_count * 1.2) + 8);
            if (rc) return rc;
        }
        uint32_t clear = sys->hstat->flags & ~FLAG_OVERFLOW;
        MDG_CUDA(cudaMemcpyAsync(&sys->dstat->flags, &clear, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        if (attempt == 3) {
            set_error("neighbour list capacity could not be sized");
            return MDG_ERR_OVERFLOW;
        }
    }
    sys->grid = *sys->hgrid;
    sys->have_list = 1;
    sys->dirty = 0;
    sys->rebuilds++;
    if (sys->hstat->build_flags & FLAG_RANGE) {
        set_error("an atom lies outside the cell grid; it was clamped into the nearest cell");
        return MDG_ERR_RANGE;
    }
    return MDG_OK;
}

}  // namespace mdg
