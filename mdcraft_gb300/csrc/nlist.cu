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

__global__ void k_grid_finalize(const double* __restrict__ part, int nparts, DomainDev d,
                                GridParams* __restrict__ out) {
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
    memset(&g, 0, sizeof(g));
    g.dim = d.dim;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < d.dim; ++i) {
        lo[i] = sh[i][0];
        hi[i] = sh[3 + i][0];
    }
    double cell = sh[6][0];
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
        *out = g;
        return;
    }
    // Grid::build (grid.cxx:43-95)
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
    if (i >= n) return;
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

__global__ void k_scan_partial(const uint32_t* __restrict__ in, int nb, uint32_t* __restrict__ bsum) {
    __shared__ uint32_t sh[32];
    int base = blockIdx.x * kScanT * kScanItems + threadIdx.x * kScanItems;
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) s += (base + k < nb) ? in[base + k] : 0u;
    uint32_t tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void k_scan_top(uint32_t* __restrict__ bsum, int nblk) {
    __shared__ uint32_t sh[32];
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

__global__ void k_scan_final(const uint32_t* __restrict__ in, int nb, const uint32_t* __restrict__ bsum,
                             uint32_t* __restrict__ out) {
    __shared__ uint32_t sh[32];
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
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[nb] = off;
}

__global__ void k_scatter(int n, const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                          const uint32_t* __restrict__ start, uint32_t* __restrict__ src) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) src[start[key[i]] + rank[i]] = (uint32_t)i;
}

// Deterministic order inside a bin: ascending caller index.
__global__ void k_bin_sort(int nb, const uint32_t* __restrict__ start, uint32_t* __restrict__ src,
                           const uint32_t* __restrict__ orig) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
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
__global__ void k_gather(int n, const uint32_t* __restrict__ src, GatherSet<NF, T> gs) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s = src[k];
#pragma unroll
    for (int f = 0; f < NF; ++f) gs.out[f][k] = gs.in[f][s];
}

// Cell centre, cell-relative FP32 offsets and packed cell of every atom.
__global__ void k_cells(int n, const double* __restrict__ rx, const double* __restrict__ ry,
                        const double* __restrict__ rz, const GridParams* __restrict__ gp,
                        uint32_t* __restrict__ cellp, double* __restrict__ Rx, double* __restrict__ Ry,
                        double* __restrict__ Rz, float4* __restrict__ pos32, float4* __restrict__ o0,
                        const uint32_t* __restrict__ orig, uint32_t* __restrict__ slot_of) {
    const GridParams g = *gp;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
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
    int n, np, K, half, uniform_rns;
    float lo2, hi2;  // rns^2 (1 -/+ 1e-5) when uniform
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
    if (warp >= g.nbins) return;
    uint32_t s0 = A.bin_start[warp], s1 = A.bin_start[warp + 1];
    if (s0 == s1) return;
    int cx, cy, cz;
    unpack_cell(A.cellp[s0], cx, cy, cz);
    int gc[3] = {cx + g.offset[0], cy + g.offset[1], cz + g.offset[2]};
    if (g.dim < 3) gc[2] = 0;
    if (g.dim < 2) gc[1] = 0;
    bool edge[3] = {false, false, false};
    for (int a = 0; a < g.dim; ++a) edge[a] = gc[a] == 0 || gc[a] == g.num[a] - 1;
    const bool prefilter = A.uniform_rns && !g.small_box;

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
                        if (prefilter && oi.w == 0.0f && oj.w == 0.0f && d2 < A.lo2) {
                            acc = true;
                        } else if (prefilter && oi.w == 0.0f && oj.w == 0.0f && d2 > A.hi2) {
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
            if (cnt > A.K) atomicOr(&A.st->flags, FLAG_OVERFLOW);
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

__global__ void k_check_rns(int n, const double* __restrict__ rns, double r0, DevStatus* st) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && rns[i] != r0) atomicOr(&st->nonuniform, 1u);
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

static int ensure_bins(mdg_system* sys, int nbins) {
    if ((size_t)nbins + 1 <= sys->bin_cap) return MDG_OK;
    size_t cap = (size_t)nbins + 1;
    cap = cap + cap / 4 + 1024;
    cudaFree(sys->bin_count);
    cudaFree(sys->bin_start);
    cudaFree(sys->scan_tmp);
    sys->bin_count = sys->bin_start = sys->scan_tmp = nullptr;
    MDG_CUDA(cudaMalloc(&sys->bin_count, cap * sizeof(uint32_t)));
    MDG_CUDA(cudaMalloc(&sys->bin_start, cap * sizeof(uint32_t)));
    MDG_CUDA(cudaMalloc(&sys->scan_tmp, (cap / (kScanT * kScanItems) + 2) * sizeof(uint32_t)));
    sys->bin_cap = cap;
    return MDG_OK;
}

static int ensure_list(mdg_system* sys, int K) {
    if (K <= sys->K && sys->nbr) return MDG_OK;
    cudaFree(sys->nbr);
    sys->nbr = nullptr;
    MDG_CUDA(cudaMalloc(&sys->nbr, (size_t)K * sys->np * sizeof(uint32_t)));
    sys->K = K;
    return MDG_OK;
}

static int launch_scan(mdg_system* sys, int nb) {
    cudaStream_t st = sys->ctx->stream;
    int nblk_scan = (nb + kScanT * kScanItems - 1) / (kScanT * kScanItems);
    if (nblk_scan > kScanT * kScanItems) {
        set_error("too many cell bins for the scan");
        return MDG_ERR_INVALID;
    }
    k_scan_partial<<<nblk_scan, kScanT, 0, st>>>(sys->bin_count, nb, sys->scan_tmp);
    MDG_LAUNCHED(sys->ctx);
    k_scan_top<<<1, kScanT, 0, st>>>(sys->scan_tmp, nblk_scan);
    MDG_LAUNCHED(sys->ctx);
    k_scan_final<<<nblk_scan, kScanT, 0, st>>>(sys->bin_count, nb, sys->scan_tmp, sys->bin_start);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

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
    int cur = sys->cur;
    if (kbuf > 0.0) {
        k_optimize_rns<<<nblk(n), kBlock, 0, st>>>(n, (int)sys->np, kbuf, sys->have_list, sys->nbr,
                                                   sys->ncnt, sys->f64[RCUT][cur], sys->f64[RNS][cur]);
        MDG_LAUNCHED(ctx);
    }
    DomainDev d;
    for (int a = 0; a < 3; ++a) {
        d.bmin[a] = sys->dom.bmin[a];
        d.bmax[a] = sys->dom.bmax[a];
        d.size[a] = sys->dom.bmax[a] - sys->dom.bmin[a];
        d.periodic[a] = sys->dom.periodic[a] ? 1 : 0;
    }
    d.dim = sys->dim;
    int nparts = std::min(nblk(n), 8 * std::max(ctx->num_sms, 1));
    if ((size_t)nparts > sys->part_cap) {
        cudaFree(sys->part);
        sys->part = nullptr;
        MDG_CUDA(cudaMalloc(&sys->part, (size_t)nparts * 8 * sizeof(double)));
        sys->part_cap = nparts;
    }
    k_wrap_bounds<<<nparts, kBlock, 0, st>>>(n, sys->f64[RX][cur], sys->f64[RY][cur], sys->f64[RZ][cur],
                                             sys->f64[RNS][cur], d, sys->part);
    MDG_LAUNCHED(ctx);
    k_grid_finalize<<<1, kBlock, 0, st>>>(sys->part, nparts, d, sys->dgrid);
    MDG_LAUNCHED(ctx);
    // uniform rns check against atom 0; per-build flags cleared
    MDG_CUDA(cudaMemsetAsync(&sys->dstat->nonuniform, 0, 2 * sizeof(uint32_t), st));
    double rns0 = 0.0;
    MDG_CUDA(cudaMemcpyAsync(&rns0, sys->f64[RNS][cur], sizeof(double), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    k_check_rns<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RNS][cur], rns0, sys->dstat);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(sys->hgrid, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    GridParams g = *sys->hgrid;
    int uniform = sys->hstat->nonuniform == 0;
    if (g.empty == -1) {
        set_error("neighbour search radius rns must be positive");
        return MDG_ERR_INVALID;
    }
    if (g.empty == -2) {
        set_error("cell grid too large (more than 1023 cells on an axis)");
        return MDG_ERR_INVALID;
    }
    sys->grid = g;
    int rc = ensure_bins(sys, g.nbins);
    if (rc) return rc;

    // bin count, scan, scatter, in-bin sort
    MDG_CUDA(cudaMemsetAsync(sys->bin_count, 0, (size_t)g.nbins * sizeof(uint32_t), st));
    k_bin_count<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RX][cur], sys->f64[RY][cur], sys->f64[RZ][cur],
                                            sys->dgrid, sys->key, sys->rank, sys->bin_count, sys->dstat);
    MDG_LAUNCHED(ctx);
    rc = launch_scan(sys, g.nbins);
    if (rc) return rc;
    k_scatter<<<nblk(n), kBlock, 0, st>>>(n, sys->key, sys->rank, sys->bin_start, sys->src);
    MDG_LAUNCHED(ctx);
    k_bin_sort<<<nblk(g.nbins), kBlock, 0, st>>>(g.nbins, sys->bin_start, sys->src, sys->u32[ORIG][cur]);
    MDG_LAUNCHED(ctx);

    // permute every per-atom field into the new slot order
    int nxt = cur ^ 1;
    {
        GatherSet<12, double> a, b;
        for (int f = 0; f < 12; ++f) {
            a.in[f] = sys->f64[f][cur];
            a.out[f] = sys->f64[f][nxt];
        }
        for (int f = 0; f < 12; ++f) {
            b.in[f] = sys->f64[12 + f][cur];
            b.out[f] = sys->f64[12 + f][nxt];
        }
        k_gather<12, double><<<nblk(n), kBlock, 0, st>>>(n, sys->src, a);
        MDG_LAUNCHED(ctx);
        k_gather<12, double><<<nblk(n), kBlock, 0, st>>>(n, sys->src, b);
        MDG_LAUNCHED(ctx);
        GatherSet<3, float> c;
        for (int f = 0; f < 3; ++f) {
            c.in[f] = sys->f32[f][cur];
            c.out[f] = sys->f32[f][nxt];
        }
        k_gather<3, float><<<nblk(n), kBlock, 0, st>>>(n, sys->src, c);
        MDG_LAUNCHED(ctx);
        GatherSet<2, uint32_t> u;
        for (int f = 0; f < 2; ++f) {
            u.in[f] = sys->u32[f][cur];
            u.out[f] = sys->u32[f][nxt];
        }
        k_gather<2, uint32_t><<<nblk(n), kBlock, 0, st>>>(n, sys->src, u);
        MDG_LAUNCHED(ctx);
        GatherSet<2, uint16_t> h;
        for (int f = 0; f < 2; ++f) {
            h.in[f] = sys->u16[f][cur];
            h.out[f] = sys->u16[f][nxt];
        }
        k_gather<2, uint16_t><<<nblk(n), kBlock, 0, st>>>(n, sys->src, h);
        MDG_LAUNCHED(ctx);
    }
    sys->cur = cur = nxt;
    k_cells<<<nblk(n), kBlock, 0, st>>>(n, sys->f64[RX][cur], sys->f64[RY][cur], sys->f64[RZ][cur], sys->dgrid,
                                        sys->cellp, sys->Rc[0], sys->Rc[1], sys->Rc[2], sys->pos32, sys->o0,
                                        sys->u32[ORIG][cur], sys->slot_of);
    MDG_LAUNCHED(ctx);

    // list capacity: estimate from the density, then grow on overflow
    if (sys->K == 0 || sys->half != half) {
        double vol = 1.0;
        for (int a = 0; a < sys->dim; ++a) vol *= g.cs[a] * g.num[a];
        double dens = (double)n / std::max(vol, 1e-300);
        double est = 4.18879020478639 * g.max_rns * g.max_rns * g.max_rns * dens;
        if (half) est *= 0.5;
        int K = (int)(est * 1.35) + 16;
        K = std::min(std::max(K, 16), n + 1);
        K = (K + 3) & ~3;
        rc = ensure_list(sys, K);
        if (rc) return rc;
    }
    double rn = g.max_rns;
    NbArgs A;
    A.n = n;
    A.np = (int)sys->np;
    A.half = half;
    A.uniform_rns = uniform;
    A.lo2 = (float)(rn * rn * (1.0 - 1e-5));
    A.hi2 = (float)(rn * rn * (1.0 + 1e-5));
    A.rx = sys->f64[RX][cur];
    A.ry = sys->f64[RY][cur];
    A.rz = sys->f64[RZ][cur];
    A.rns = sys->f64[RNS][cur];
    A.rcut = sys->f64[RCUT][cur];
    A.orig = sys->u32[ORIG][cur];
    A.uid = sys->u32[UID][cur];
    A.cellp = sys->cellp;
    A.bin_start = sys->bin_start;
    A.o0 = sys->o0;
    A.ncnt = sys->ncnt;
    A.r0x = sys->r0[0];
    A.r0y = sys->r0[1];
    A.r0z = sys->r0[2];
    A.saved_rcut = sys->saved_rcut;
    A.saved_rns = sys->saved_rns;
    A.saved_uid = sys->saved_uid;
    A.st = sys->dstat;
    for (int attempt = 0; attempt < 3; ++attempt) {
        A.K = sys->K;
        A.nbr = sys->nbr;
        MDG_CUDA(cudaMemsetAsync(&sys->dstat->max_count, 0, sizeof(uint32_t), st));
        int warps = g.nbins;
        k_nbuild<<<nblk((size_t)warps * 32), kBlock, 0, st>>>(A, sys->dgrid);
        MDG_LAUNCHED(ctx);
        MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
        MDG_CUDA(cudaStreamSynchronize(st));
        uint32_t mc = sys->hstat->max_count;
        if ((int)mc <= sys->K) break;
        int K = (int)(mc * 1.2) + 8;
        K = (K + 3) & ~3;
        rc = ensure_list(sys, K);
        if (rc) return rc;
        // overflow of this attempt is resolved by the retry
        uint32_t clear = sys->hstat->flags & ~FLAG_OVERFLOW;
        MDG_CUDA(cudaMemcpyAsync(&sys->dstat->flags, &clear, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    }
    sys->have_list = 1;
    sys->half = half;
    sys->dirty = 0;
    sys->rebuilds++;
    if (sys->hstat->build_flags & FLAG_RANGE) {
        set_error("an atom lies outside the cell grid; it was clamped into the nearest cell");
        return MDG_ERR_RANGE;
    }
    return MDG_OK;
}

}  // namespace mdg
