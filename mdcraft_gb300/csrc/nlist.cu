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

#include "mdg_host.h"

namespace mdg {

// ---------------------------------------------------------------------------
// bounds + wrap (Domain::fit_in_period, domain.cxx:41-47; Grid::find_bounds,
// grid.cxx:209-243)
// ---------------------------------------------------------------------------
struct DomainDev {
    double bmin[3], bmax[3], size[3];
    int periodic[3];
    int dim;
};

__global__ void k_wrap_bounds(int n, double* __restrict__ rx, double* __restrict__ ry,
                              double* __restrict__ rz, const double* __restrict__ rns,
                              DomainDev d, double* __restrict__ part) {
    __shared__ double sh[7][kBlock];
    double lo[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double hi[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    double mr = 0.0;
    double* r[3] = {rx, ry, rz};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int a = 0; a < 3; ++a) {
            double v = r[a][i];
            if (d.periodic[a]) {
                double w = v < d.bmin[a] ? dadd(v, d.size[a]) : v > d.bmax[a] ? dsub(v, d.size[a]) : v;
                if (w != v) r[a][i] = w;
                v = w;
            }
            lo[a] = fmin(lo[a], v);
            hi[a] = fmax(hi[a], v);
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

// Grid::build (grid.cxx:43-95) from the reduced bounds and the largest rns;
// shared by the device rebuild and the host-side capacity sizing, so both
// get the same parameters bit for bit.
__host__ __device__ void grid_from_bounds(const DomainDev& d, const double lo_in[3], const double hi_in[3],
                                          double cell, GridParams& g) {
    memset(&g, 0, sizeof(g));
    g.dim = d.dim;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < d.dim; ++i) {
        lo[i] = lo_in[i];
        hi[i] = hi_in[i];
    }
    g.max_rns = cell;
    for (int i = 0; i < 3; ++i) {
        g.bmin[i] = d.bmin[i];
        g.bmax[i] = d.bmax[i];
        g.size[i] = d.size[i];
        g.periodic[i] = d.periodic[i];
        g.dom_n[i] = 1;
        g.cs[i] = d.size[i];
    }
    if (!(cell > 0.0)) {
        g.empty = -1;
        return;
    }
    for (int i = 0; i < d.dim; ++i) {
        double q = floor(d.size[i] / cell);
        int c = q > 1.0e9 ? 1000000000 : (int)q;
        g.dom_n[i] = c > 1 ? c : 1;
    }
    for (int i = 0; i < d.dim; ++i) g.cs[i] = d.size[i] / (double)g.dom_n[i];
    int up[3] = {0, 0, 0};
    for (int i = 0; i < d.dim; ++i) {
        g.offset[i] = (int)floor((lo[i] - d.bmin[i]) / g.cs[i]);
        up[i] = (int)floor((hi[i] - d.bmin[i]) / g.cs[i]);
        int u = up[i] + 1;
        up[i] = u < g.dom_n[i] ? u : g.dom_n[i];
    }
    for (int i = 0; i < 3; ++i) g.num[i] = 1;
    for (int i = 0; i < d.dim; ++i) g.num[i] = up[i] - g.offset[i];
    g.small_box = 0;
    for (int i = 0; i < 3; ++i) {
        g.gmin[i] = d.bmin[i];
        if (i < d.dim) g.gmin[i] = d.bmin[i] + g.cs[i] * g.offset[i];
        g.bricks[i] = (g.num[i] + 3) / 4;
        g.csf[i] = (float)g.cs[i];
        g.Lf[i] = (float)d.size[i];
        if (d.periodic[i] && i < d.dim &&
            (g.dom_n[i] <= 3 || g.offset[i] != 0 || g.num[i] != g.dom_n[i]))
            g.small_box = 1;
        if (g.num[i] < 1 || g.num[i] > 1023) g.empty = -2;
    }
    long long nc = (long long)g.num[0] * g.num[1] * g.num[2];
    long long nb = 64LL * g.bricks[0] * g.bricks[1] * g.bricks[2];
    if (nb > (1LL << 30)) g.empty = -2;
    g.ncells = (int)nc;
    g.nbins = (int)nb;
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
__device__ __forceinline__ void local_cell(const GridParams& g, double x, double y, double z,
                                           int c[3], bool& clamped) {
    double r[3] = {x, y, z};
    clamped = false;
    for (int a = 0; a < 3; ++a) {
        int v = 0;
        if (a < g.dim) v = (int)floor(__ddiv_rn(dsub(r[a], g.bmin[a]), g.cs[a])) - g.offset[a];
        if (v < 0) { v = 0; clamped = true; }
        if (v >= g.num[a]) { v = g.num[a] - 1; clamped = true; }
        c[a] = v;
    }
}

__global__ void k_bin_count(int n, const double* __restrict__ rx, const double* __restrict__ ry,
                            const double* __restrict__ rz, const GridParams* __restrict__ gp,
                            uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                            uint32_t* __restrict__ bin_count, DevStatus* st) {
    const GridParams g = *gp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || g.empty) return;
    int c[3];
    bool cl;
    local_cell(g, rx[i], ry[i], rz[i], c, cl);
    if (cl) {
        atomicOr(&st->flags, FLAG_RANGE);
        atomicOr(&st->build_flags, FLAG_RANGE);
    }
    uint32_t k = (uint32_t)bin_key(g, c[0], c[1], c[2]);
    key[i] = k;
    rank[i] = atomicAdd(&bin_count[k], 1u);
}

// Exclusive scan of nb uint32 counts into start[0..nb] (start[nb] = total),
// 4096 items per block: per-block totals, a one-block scan of the totals,
// then per-block scans with offsets.
constexpr int kScanT = 1024, kScanItems = 4;

__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* sh, uint32_t* total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        sh[lane] = s;
    }
    __syncthreads();
    uint32_t base = w > 0 ? sh[w - 1] : 0u;
    uint32_t tot = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    if (total) *total = tot;
    return base + x - v;
}

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
    uint32_t s = start[b], e = start[b + 1];
    for (uint32_t k = s + 1; k < e; ++k) {
        uint32_t v = src[k];
        uint32_t ov = orig[v];
        uint32_t m = k;
        while (m > s && orig[src[m - 1]] > ov) {
            src[m] = src[m - 1];
            --m;
        }
        src[m] = v;
    }
}

// Permutation of the per-atom fields: dst[k] = src_field[src[k]].
template <int NF, typename T>
struct GatherSet {
    const T* in[NF];
    T* out[NF];
};

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
                        double* __restrict__ Rz, float4* __restrict__ pos32, float4* __restrict__ o0,
                        const uint32_t* __restrict__ orig, uint32_t* __restrict__ slot_of) {
    const GridParams g = *gp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || g.empty) return;
    double r[3] = {rx[i], ry[i], rz[i]};
    int c[3];
    bool cl;
    local_cell(g, r[0], r[1], r[2], c, cl);
    cellp[i] = pack_cell(c[0], c[1], c[2]);
    double R[3];
    float o[3];
    bool outlier = cl;
    for (int a = 0; a < 3; ++a) {
        R[a] = g.gmin[a] + ((double)c[a] + 0.5) * g.cs[a];
        if (a >= g.dim) R[a] = r[a];
        o[a] = (float)(r[a] - R[a]);
        if (fabsf(o[a]) > 0.75f * g.csf[a] && a < g.dim) outlier = true;
    }
    Rx[i] = R[0];
    Ry[i] = R[1];
    Rz[i] = R[2];
    float4 p = make_float4(o[0], o[1], o[2], 0.0f);
    pos32[i] = p;
    o0[i] = make_float4(o[0], o[1], o[2], outlier ? 1.0f : 0.0f);
    slot_of[orig[i]] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// Verlet list: one warp per cell, lanes over the cell's atoms
// ---------------------------------------------------------------------------
struct NbArgs {
    int n, np, K, half;
    const double *rx, *ry, *rz, *rns, *rcut;
    const uint32_t *orig, *uid, *cellp, *bin_start;
    const float4* o0;
    uint32_t *nbr, *ncnt;
    double *r0x, *r0y, *r0z, *saved_rcut, *saved_rns;
    uint32_t* saved_uid;
    DevStatus* st;
};

// VerletList::are_neibs (verlet-list.cxx:373-400), FP64 without contraction.
__device__ __forceinline__ bool are_neibs_exact(const GridParams& g, double xa, double ya, double za,
                                                double ra, double xb, double yb, double zb, double rb,
                                                const bool edge[3]) {
    double dd = ra < rb ? rb : ra;
    double d2 = dmul(dd, dd);
    double drx = dsub(xa, xb), dry = dsub(ya, yb), drz = dsub(za, zb);
    double xs = g.size[0], ys = g.size[1], zs = g.size[2];
    if (edge[0] && g.periodic[0] && (2 * drx < -xs)) drx = dadd(drx, xs);
    if (edge[0] && g.periodic[0] && (2 * drx > xs)) drx = dsub(drx, xs);
    if (edge[1] && g.periodic[1] && (2 * dry < -ys)) dry = dadd(dry, ys);
    if (edge[1] && g.periodic[1] && (2 * dry > ys)) dry = dsub(dry, ys);
    if (edge[2] && g.periodic[2] && (2 * drz < -zs)) drz = dadd(drz, zs);
    if (edge[2] && g.periodic[2] && (2 * drz > zs)) drz = dsub(drz, zs);
    return sq3_exact(drx, dry, drz) <= d2;
}

__global__ void __launch_bounds__(kBlock) k_nbuild(NbArgs A, const GridParams* __restrict__ gp) {
    __shared__ GridParams g;
    if (threadIdx.x == 0) g = *gp;
    __syncthreads();
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (g.empty || warp >= g.nbins) return;
    // prefilter band: rns^2 (1 -/+ 1e-5), valid when every atom has the same rns
    const float lo2 = (float)(g.max_rns * g.max_rns * (1.0 - 1e-5));
    const float hi2 = (float)(g.max_rns * g.max_rns * (1.0 + 1e-5));
    const bool uniform_rns = A.st->nonuniform == 0;
    uint32_t s0 = A.bin_start[warp], s1 = A.bin_start[warp + 1];
    if (s0 == s1) return;
    int cx, cy, cz;
    unpack_cell(A.cellp[s0], cx, cy, cz);
    int gc[3] = {cx + g.offset[0], cy + g.offset[1], cz + g.offset[2]};
    if (g.dim < 3) gc[2] = 0;
    if (g.dim < 2) gc[1] = 0;
    bool edge[3] = {false, false, false};
    for (int a = 0; a < g.dim; ++a) edge[a] = gc[a] == 0 || gc[a] == g.num[a] - 1;
    const bool prefilter = uniform_rns && !g.small_box;

    for (uint32_t base = s0; base < s1; base += 32) {
        uint32_t i = base + lane;
        bool active = i < s1;
        double xi = 0, yi = 0, zi = 0, rni = 0;
        float4 oi = make_float4(0, 0, 0, 0);
        uint32_t origi = 0;
        if (active) {
            xi = A.rx[i]; yi = A.ry[i]; zi = A.rz[i]; rni = A.rns[i];
            oi = A.o0[i];
            origi = A.orig[i];
        }
        int cnt = 0;
        for (int x = -1; x <= 1; ++x) {
            if (g.periodic[0]) {
                if (g.dom_n[0] == 1 && x != 0) continue;
                if (g.dom_n[0] == 2 && x == 1) continue;
            }
            for (int y = -1; y <= 1; ++y) {
                if (g.periodic[1]) {
                    if (g.dom_n[1] == 1 && y != 0) continue;
                    if (g.dom_n[1] == 2 && y == 1) continue;
                }
                for (int z = -1; z <= 1; ++z) {
                    if (g.periodic[2]) {
                        if (g.dom_n[2] == 1 && z != 0) continue;
                        if (g.dom_n[2] == 2 && z == 1) continue;
                    }
                    int nb[3] = {gc[0] + x, gc[1] + y, gc[2] + z};
                    for (int a = 0; a < 3; ++a)
                        if (g.periodic[a]) nb[a] = (nb[a] + g.dom_n[a]) % g.dom_n[a];
                    int lc[3] = {nb[0] - g.offset[0], nb[1] - g.offset[1], nb[2] - g.offset[2]};
                    if (lc[0] < 0 || lc[0] >= g.num[0] || lc[1] < 0 || lc[1] >= g.num[1] ||
                        lc[2] < 0 || lc[2] >= g.num[2])
                        continue;
                    int bk = bin_key(g, lc[0], lc[1], lc[2]);
                    uint32_t j0 = A.bin_start[bk], j1 = A.bin_start[bk + 1];
                    // image of the neighbour cell relative to this cell
                    int dl[3] = {x, y, z};
                    float sh[3] = {(float)x * g.csf[0], (float)y * g.csf[1], (float)z * g.csf[2]};
                    for (uint32_t j = j0; j < j1; ++j) {
                        float4 oj = A.o0[j];
                        if (!active || j == i) continue;
                        if (A.half && A.orig[j] < origi) continue;
                        float dx = oi.x - oj.x - sh[0];
                        float dy = oi.y - oj.y - sh[1];
                        float dz = oi.z - oj.z - sh[2];
                        float d2 = dx * dx + dy * dy + dz * dz;
                        bool acc;
                        if (prefilter && oi.w == 0.0f && oj.w == 0.0f && d2 < lo2) {
                            acc = true;
                        } else if (prefilter && oi.w == 0.0f && oj.w == 0.0f && d2 > hi2) {
                            acc = false;
                        } else {
                            acc = are_neibs_exact(g, xi, yi, zi, rni, A.rx[j], A.ry[j], A.rz[j],
                                                  A.rns[j], edge);
                        }
                        if (!acc) continue;
                        // periodic image code: minimum image of j seen from i
                        uint32_t code = 0;
                        for (int a = 0; a < 3; ++a) {
                            int dlt = dl[a];
                            if (g.periodic[a] && a < g.dim && g.dom_n[a] <= 3) {
                                float dd = -(a == 0 ? dx : a == 1 ? dy : dz);
                                float half = 0.5f * g.Lf[a];
                                if (dd > half) dlt -= g.dom_n[a];
                                else if (dd < -half) dlt += g.dom_n[a];
                            }
                            if (dlt < -1 || dlt > 1) {
                                atomicOr(&A.st->flags, FLAG_IMAGE);
                                dlt = dlt < -1 ? -1 : 1;
                            }
                            code |= (uint32_t)(dlt + 1) << (2 * a);
                            // the image crossed a periodic face
                            int own[3] = {cx, cy, cz};
                            if (dlt != lc[a] - own[a]) code |= 1u << 6;
                        }
                        if (cnt < A.K) A.nbr[nidx(cnt, i, A.np)] = j | (code << kJBits);
                        ++cnt;
                    }
                }
            }
        }
        if (active) {
            // pad to a multiple of four with self entries
            int padded = (cnt + 3) & ~3;
            for (int k = cnt; k < padded && k < A.K; ++k) A.nbr[nidx(k, i, A.np)] = i | kSelfCode;
            A.ncnt[i] = padded < A.K ? padded : A.K;
            if (cnt > A.K) {
                atomicOr(&A.st->flags, FLAG_OVERFLOW);
                atomicOr(&A.st->build_flags, FLAG_OVERFLOW);
            }
            atomicMax(&A.st->max_count, (uint32_t)cnt);
            A.r0x[i] = xi;
            A.r0y[i] = yi;
            A.r0z[i] = zi;
            A.saved_rcut[i] = A.rcut[i];
            A.saved_rns[i] = rni;
            A.saved_uid[i] = A.uid[i];
        }
    }
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
int nlist_enqueue(mdg_system* sys) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)sys->n;
    if (n == 0) return MDG_OK;
    int nparts = nparts_of(sys);
    DomainDev d = domain_dev(sys);
    const int c = sys->cur, alt = c ^ 1;
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
        GatherSet<12, double> a, b, a2, b2;
        for (int f = 0; f < 12; ++f) {
            a.in[f] = sys->f64[f][c];
            a.out[f] = sys->f64[f][alt];
            b.in[f] = sys->f64[12 + f][c];
            b.out[f] = sys->f64[12 + f][alt];
            a2.in[f] = a.out[f];
            a2.out[f] = sys->f64[f][c];
            b2.in[f] = b.out[f];
            b2.out[f] = sys->f64[12 + f][c];
        }
        GatherSet<3, float> fc, fc2;
        for (int f = 0; f < 3; ++f) {
            fc.in[f] = sys->f32[f][c];
            fc.out[f] = sys->f32[f][alt];
            fc2.in[f] = fc.out[f];
            fc2.out[f] = sys->f32[f][c];
        }
        GatherSet<2, uint32_t> u, u2;
        GatherSet<2, uint16_t> h, h2;
        for (int f = 0; f < 2; ++f) {
            u.in[f] = sys->u32[f][c];
            u.out[f] = sys->u32[f][alt];
            u2.in[f] = u.out[f];
            u2.out[f] = sys->u32[f][c];
            h.in[f] = sys->u16[f][c];
            h.out[f] = sys->u16[f][alt];
            h2.in[f] = h.out[f];
            h2.out[f] = sys->u16[f][c];
        }
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
                                        sys->cellp, sys->Rc[0], sys->Rc[1], sys->Rc[2], sys->pos32, sys->o0,
                                        sys->u32[ORIG][c], sys->slot_of);
    MDG_LAUNCHED(ctx);
    NbArgs A;
    A.n = n;
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
    size_t warps = sys->bin_cap;  // one warp per bin; the live bins come from the device grid
    k_nbuild<<<nblk(warps * 32), kBlock, 0, st>>>(A, sys->dgrid);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
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
