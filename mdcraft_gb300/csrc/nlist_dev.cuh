// nlist_dev.cuh — device pieces of the linked-cell rebuild and the Verlet
// list build, shared by the per-stage kernels (nlist.cu) and the fused
// per-system loop (solo.cu) so both compute the same lists bit for bit.
//
// Grid::build / local_index3D / adjacent_cells (mdcraft/neibs/grid.cxx:43-207),
// Domain::fit_in_period (mdcraft/lattice/domain.cxx:41-47) and
// VerletList::build_linked_cells / are_neibs
// (mdcraft/neibs/verlet-list.cxx:306-400).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "mdg_internal.cuh"

namespace mdg {

// ---- bounds + wrap ----------------------------------------------------------
struct DomainDev {
    double bmin[3], bmax[3], size[3];
    int periodic[3];
    int dim;
};

// Grid::build (grid.cxx:43-95) from the reduced bounds and the largest rns;
// shared by the device rebuild and the host-side capacity sizing, so both
// get the same parameters bit for bit.
__host__ __device__ inline void grid_from_bounds(const DomainDev& d, const double lo_in[3], const double hi_in[3],
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
        g.inv_u[i] = g.cs[i] > 0.0 ? kOffUnits / g.cs[i] : 0.0;
        g.inv_cs[i] = g.cs[i] > 0.0 ? 1.0 / g.cs[i] : 0.0;
        // A periodic axis of 3 cells keeps the fast paths: its cells are at
        // least max rns wide (floor(L / rns) = 3), so every listed pair is
        // nearer than L / 2 and the image of its neighbour cell is the
        // minimum image (no per-pair adjustment, the FP32 prefilter holds).
        // One or two cells per axis (the reference's n = 1, 2 rules), or a
        // local grid short of the periodic box, take the per-atom body,
        // whose prefilter takes a per-pair minimum image.
        if (d.periodic[i] && i < d.dim &&
            (g.dom_n[i] <= 2 || g.offset[i] != 0 || g.num[i] != g.dom_n[i]))
            g.small_box = 1;
        if (g.num[i] < 1 || g.num[i] > 1023) g.empty = -2;
    }
    long long nc = (long long)g.num[0] * g.num[1] * g.num[2];
    long long nb = 64LL * g.bricks[0] * g.bricks[1] * g.bricks[2];
    if (nb > (1LL << 30)) g.empty = -2;
    g.ncells = (int)nc;
    g.nbins = (int)nb;
}

// floor(x / cs) with the quotient correctly rounded in FP64, as the
// reference's cell index takes it (grid.cxx). The product with the
// reciprocal 1/cs (itself rounded) lies within 1.5 * 2^-52 (relative) of the
// exact quotient, as does the rounded quotient, so the two have the same
// floor unless an integer lies within that distance of the product. Below
// 2^20 cells that distance is under 3.5e-10: a product within 1e-9 of an
// integer, or beyond 2^20, takes the division instead.
__device__ __forceinline__ int floor_div(double x, double cs, double inv_cs) {
    const double q = dmul(x, inv_cs);
    const double f = floor(q);
    const double frac = dsub(q, f);  // exact: f <= q < f + 1
    if (frac > 1e-9 && frac < 1.0 - 1e-9 && fabs(q) < 1048576.0) return (int)f;
    return (int)floor(__ddiv_rn(x, cs));
}

__device__ __forceinline__ void local_cell(const GridParams& g, double x, double y, double z,
                                           int c[3], bool& clamped) {
    double r[3] = {x, y, z};
    clamped = false;
    for (int a = 0; a < 3; ++a) {
        int v = 0;
        if (a < g.dim) v = floor_div(dsub(r[a], g.bmin[a]), g.cs[a], g.inv_cs[a]) - g.offset[a];
        if (v < 0) { v = 0; clamped = true; }
        if (v >= g.num[a]) { v = g.num[a] - 1; clamped = true; }
        c[a] = v;
    }
}

__device__ inline uint32_t block_excl_scan(uint32_t v, uint32_t* sh, uint32_t* total) {
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

template <int NF, typename T>
struct GatherSet {
    const T* in[NF];
    T* out[NF];
};

// Positions wrapped into the box on periodic axes (Domain::fit_in_period),
// written back; returns the wrapped position for the bounds.
__device__ __forceinline__ void wrap_one(const DomainDev& d, double* rx, double* ry, double* rz, int i,
                                         double v[3]) {
    double* r[3] = {rx, ry, rz};
    for (int a = 0; a < 3; ++a) {
        double x = r[a][i];
        if (d.periodic[a]) {
            double w = x < d.bmin[a] ? dadd(x, d.size[a]) : x > d.bmax[a] ? dsub(x, d.size[a]) : x;
            if (w != x) r[a][i] = w;
            x = w;
        }
        v[a] = x;
    }
}

// Bin key of atom i and its arrival rank in the bin.
__device__ __forceinline__ void bin_count_one(const GridParams& g, int i, const double* rx, const double* ry,
                                              const double* rz, uint32_t* key, uint32_t* rank,
                                              uint32_t* bin_count, DevStatus* st) {
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

// Deterministic order inside bin b: ascending caller index.
__device__ __forceinline__ void bin_sort_one(int b, const uint32_t* start, uint32_t* src, const uint32_t* orig) {
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

// Cell centre, cell-relative FP32 offsets and packed cell of atom i.
__device__ __forceinline__ void cells_one(const GridParams& g, int i, const double* rx, const double* ry,
                                          const double* rz, uint32_t* cellp, double* Rx, double* Ry, double* Rz,
                                          int4* pos32, int4* q0, float4* o0, const uint32_t* orig,
                                          uint32_t* slot_of, const uint16_t* kind) {
    double r[3] = {rx[i], ry[i], rz[i]};
    int c[3];
    bool cl;
    local_cell(g, r[0], r[1], r[2], c, cl);
    cellp[i] = pack_cell(c[0], c[1], c[2]);
    double R[3];
    float o[3];
    int q[3];
    bool outlier = cl;
    for (int a = 0; a < 3; ++a) {
        R[a] = g.gmin[a] + ((double)c[a] + 0.5) * g.cs[a];
        if (a >= g.dim) R[a] = r[a];
        o[a] = (float)(r[a] - R[a]);
        q[a] = off_encode(r[a] - R[a], g.inv_u[a]);
        if (fabsf(o[a]) > 0.75f * g.csf[a] && a < g.dim) outlier = true;
    }
    Rx[i] = R[0];
    Ry[i] = R[1];
    Rz[i] = R[2];
    pos32[i] = make_int4(q[0], q[1], q[2], kind[i] & 3);  // w: the atom's kind (Multi passes)
    q0[i] = make_int4(q[0], q[1], q[2], 0);
    // w: 0 exact offsets; 1 not exact (the FP32 tests send its pairs to FP64);
    // 2 clamped into the grid (also not exact: its list is walked from the
    // unclamped cell, nbuild_atom)
    o0[i] = make_float4(o[0], o[1], o[2], cl ? 2.0f : outlier ? 1.0f : 0.0f);
    slot_of[orig[i]] = (uint32_t)i;
}

// Every permuted field of one rebuild: the gathers into the spare buffers
// and the copies back.
struct GatherAll {
    GatherSet<12, double> a, b, a2, b2;
    GatherSet<3, float> fc, fc2;
    GatherSet<2, uint32_t> u, u2;
    GatherSet<2, uint16_t> h, h2;
};

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

// The grid covers every cell of each periodic axis (no local grid short of
// the box).
__device__ __forceinline__ bool grid_whole(const GridParams& g) {
    for (int a = 0; a < g.dim; ++a)
        if (g.periodic[a] && (g.offset[a] != 0 || g.num[a] != g.dom_n[a])) return false;
    return true;
}

// Image code of a listed pair (list entry bits above kJBits): per axis the
// cell offset of j's image seen from i's cell (own), from the neighbour
// cell's offset dl, moved by a period on axes of 3 cells or fewer when the
// FP32 displacement (dx, dy, dz: i minus the neighbour cell's image of j)
// says the other image is nearer; bit 6 when the image crossed a periodic
// face (the offset differs from the local cells' difference lc - own).
__device__ __forceinline__ uint32_t pair_image_code(const GridParams& g, const int own[3], const int lc[3],
                                                    const int dl[3], float dx, float dy, float dz,
                                                    DevStatus* st) {
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
            atomicOr(&st->flags, FLAG_IMAGE);
            dlt = dlt < -1 ? -1 : 1;
        }
        code |= (uint32_t)(dlt + 1) << (2 * a);
        if (dlt != lc[a] - own[a]) code |= 1u << 6;
    }
    return code;
}

// The nearest image of a displacement d on a periodic axis of length L,
// for |d| < 1.5 L (the offsets of binned atoms are within half a cell of
// their cell centres, so one shift suffices on axes of one or two cells).
__device__ __forceinline__ float min_image_f(float d, float L) {
    const float half = 0.5f * L;
    if (d > half) return d - L;
    if (d < -half) return d + L;
    return d;
}

// The list of atom i (one thread per atom, over the whole grid: used for
// grids with a periodic axis of 2 cells or fewer, which have few cells of
// many atoms each): its cell's 27 (or fewer, on small periodic axes)
// neighbour cells in the reference's order, x outer, z inner, each cell's
// atoms in slot order. The FP32 prefilter also holds on periodic axes of
// one or two cells when the grid covers the whole box: every cell there is
// an edge cell, so the exact test takes the minimum image, and the FP32
// minimum image of the neighbour cell's displacement is the same distance
// to ~1e-6 of r^2, inside the band that goes to FP64. A local grid short of
// the box keeps the FP64 test for every candidate.
// An atom clamped into the grid (a position on the upper face of a periodic
// axis after the wrap, or outside the grid) is binned in its clamped cell,
// but, as Grid::adjacent_cells (grid.cxx:138-207) takes the cell of the
// position itself, its own walk and edge flags come from the unclamped cell;
// the image codes stay relative to the cell it is binned in.
__device__ __forceinline__ void nbuild_atom(const NbArgs& A, const GridParams& g, uint32_t i, bool uniform_rns) {
    // prefilter band: rns^2 (1 -/+ 1e-5), valid when every atom has the same rns
    const float lo2 = (float)(g.max_rns * g.max_rns * (1.0 - 1e-5));
    const float hi2 = (float)(g.max_rns * g.max_rns * (1.0 + 1e-5));
    int cx, cy, cz;
    unpack_cell(A.cellp[i], cx, cy, cz);
    const int own[3] = {cx, cy, cz};
    const double xi = A.rx[i], yi = A.ry[i], zi = A.rz[i], rni = A.rns[i];
    const float4 oi = A.o0[i];
    // the walk's cell (global index) and its offset from the binned cell
    int gc[3] = {cx + g.offset[0], cy + g.offset[1], cz + g.offset[2]};
    int shift[3] = {0, 0, 0};
    if (oi.w == 2.0f) {
        const double r[3] = {xi, yi, zi};
        for (int a = 0; a < g.dim; ++a) {
            const int u = floor_div(dsub(r[a], g.bmin[a]), g.cs[a], g.inv_cs[a]);
            shift[a] = u - gc[a];
            gc[a] = u;
        }
    }
    if (g.dim < 3) gc[2] = 0;
    if (g.dim < 2) gc[1] = 0;
    bool edge[3] = {false, false, false};
    for (int a = 0; a < g.dim; ++a) edge[a] = gc[a] == 0 || gc[a] == g.num[a] - 1;
    bool mi[3] = {false, false, false};
    for (int a = 0; a < g.dim; ++a) mi[a] = g.periodic[a] && g.dom_n[a] <= 2;
    const bool prefilter = uniform_rns && grid_whole(g);
    const uint32_t origi = A.orig[i];
    const bool pfi = prefilter && oi.w == 0.0f;
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
                int lc[3];
                bool inside = true;
                for (int a = 0; a < 3; ++a) {
                    // the walk's cell is within one cell of the grid, so one period at most
                    int nb = gc[a] + (a == 0 ? x : a == 1 ? y : z);
                    if (g.periodic[a]) nb = nb < 0 ? nb + g.dom_n[a] : nb >= g.dom_n[a] ? nb - g.dom_n[a] : nb;
                    lc[a] = nb - g.offset[a];
                    inside = inside && lc[a] >= 0 && lc[a] < g.num[a];
                }
                if (!inside) continue;
                const int bk = bin_key(g, lc[0], lc[1], lc[2]);
                const uint32_t j0 = A.bin_start[bk], j1 = A.bin_start[bk + 1];
                // image of the neighbour cell relative to the binned cell
                const int dl[3] = {x + shift[0], y + shift[1], z + shift[2]};
                const float sh[3] = {(float)dl[0] * g.csf[0], (float)dl[1] * g.csf[1], (float)dl[2] * g.csf[2]};
                for (uint32_t j = j0; j < j1; ++j) {
                    if (j == i) continue;
                    if (A.half && A.orig[j] < origi) continue;
                    const float4 oj = A.o0[j];
                    const float dx = oi.x - oj.x - sh[0];
                    const float dy = oi.y - oj.y - sh[1];
                    const float dz = oi.z - oj.z - sh[2];
                    const float ex = mi[0] ? min_image_f(dx, g.Lf[0]) : dx;
                    const float ey = mi[1] ? min_image_f(dy, g.Lf[1]) : dy;
                    const float ez = mi[2] ? min_image_f(dz, g.Lf[2]) : dz;
                    const float d2 = ex * ex + ey * ey + ez * ez;
                    bool acc;
                    if (pfi && oj.w == 0.0f && d2 < lo2) acc = true;
                    else if (pfi && oj.w == 0.0f && d2 > hi2) acc = false;
                    else acc = are_neibs_exact(g, xi, yi, zi, rni, A.rx[j], A.ry[j], A.rz[j], A.rns[j], edge);
                    if (!acc) continue;
                    // periodic image code: minimum image of j seen from i
                    const uint32_t code = pair_image_code(g, own, lc, dl, dx, dy, dz, A.st);
                    if (cnt < A.K) A.nbr[nidx(cnt, i, A.np)] = j | (code << kJBits);
                    ++cnt;
                }
            }
        }
    }
    // pad to a multiple of four with self entries
    const int padded = (cnt + 3) & ~3;
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

// ---- list build, a warp per cell with lanes over candidates -------------------
// The cell's candidates are the atoms of its neighbour cells in the
// reference's cell order (x outer, z inner), each cell's atoms in slot order.
// Lanes take 32 consecutive candidates; the warp walks the cell's atoms, one
// ballot per atom, so lane i ends with atom i's row of the chunk's accept
// matrix and appends those candidates in lane order.
// Entry order per atom is therefore the order of the per-atom loop in
// nbuild_atom, and the lists are the same, entry for entry. Used when no
// periodic axis has 2 cells or fewer (no minimum-image adjustment of the
// image code, GridParams::small_box); otherwise nbuild_atom runs.
struct NbWarpSmem {
    uint32_t cj0[27];        // first slot of each non-empty neighbour cell
    uint32_t cpre[28];       // candidate prefix over those cells
    uint32_t ccode[27];      // image code << kJBits
    float4 csh[27];          // cell shift (x, y, z) of the image
    float4 oi[32];           // the batch's offsets
    uint32_t origi[32];
    uint32_t cand[32];       // the chunk's list entries (slot | image code)
};

__device__ __forceinline__ void nbuild_cell_warp(const NbArgs& A, const GridParams& g, int bin, int lane,
                                                 bool uniform_rns, NbWarpSmem& S) {
    const unsigned full = 0xffffffffu;
    const float lo2 = (float)(g.max_rns * g.max_rns * (1.0 - 1e-5));
    const float hi2 = (float)(g.max_rns * g.max_rns * (1.0 + 1e-5));
    const uint32_t s0 = A.bin_start[bin], s1 = A.bin_start[bin + 1];
    if (s0 == s1) return;
    int cx, cy, cz;
    unpack_cell(A.cellp[s0], cx, cy, cz);
    int gc[3] = {cx + g.offset[0], cy + g.offset[1], cz + g.offset[2]};
    if (g.dim < 3) gc[2] = 0;
    if (g.dim < 2) gc[1] = 0;
    bool edge[3] = {false, false, false};
    for (int a = 0; a < g.dim; ++a) edge[a] = gc[a] == 0 || gc[a] == g.num[a] - 1;

    // lane t < 27: neighbour cell (t / 9 - 1, t / 3 % 3 - 1, t % 3 - 1)
    bool valid = false;
    uint32_t j0 = 0, ncand = 0, code = 0;
    float4 sh = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < 27) {
        const int dl[3] = {lane / 9 - 1, (lane / 3) % 3 - 1, lane % 3 - 1};
        valid = true;
        for (int a = 0; a < 3; ++a)
            if (g.periodic[a] && ((g.dom_n[a] == 1 && dl[a] != 0) || (g.dom_n[a] == 2 && dl[a] == 1))) valid = false;
        if (valid) {
            int nb[3] = {gc[0] + dl[0], gc[1] + dl[1], gc[2] + dl[2]};
            for (int a = 0; a < 3; ++a)
                if (g.periodic[a]) nb[a] = (nb[a] + g.dom_n[a]) % g.dom_n[a];
            const int lc[3] = {nb[0] - g.offset[0], nb[1] - g.offset[1], nb[2] - g.offset[2]};
            if (lc[0] < 0 || lc[0] >= g.num[0] || lc[1] < 0 || lc[1] >= g.num[1] || lc[2] < 0 || lc[2] >= g.num[2]) {
                valid = false;
            } else {
                const int bk = bin_key(g, lc[0], lc[1], lc[2]);
                j0 = A.bin_start[bk];
                ncand = A.bin_start[bk + 1] - j0;
                sh = make_float4((float)dl[0] * g.csf[0], (float)dl[1] * g.csf[1], (float)dl[2] * g.csf[2], 0.f);
                const int own[3] = {cx, cy, cz};
                for (int a = 0; a < 3; ++a) {
                    code |= (uint32_t)(dl[a] + 1) << (2 * a);
                    if (dl[a] != lc[a] - own[a]) code |= 1u << 6;  // the image crossed a periodic face
                }
            }
        }
    }
    const bool use = valid && ncand > 0;
    const unsigned vm = __ballot_sync(full, use);
    const int slot = __popc(vm & ((1u << lane) - 1u));
    const int nc = __popc(vm);
    uint32_t incl = use ? ncand : 0u;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += v;
    }
    if (use) {
        S.cj0[slot] = j0;
        S.cpre[slot] = incl - ncand;
        S.ccode[slot] = code << kJBits;
        S.csh[slot] = sh;
    }
    const uint32_t T = __shfl_sync(full, incl, 31);
    if (lane == 0) S.cpre[nc] = T;
    // the cell itself (lane 13: offset (0, 0, 0)) among the used cells
    const int home = __popc(vm & ((1u << 13) - 1u));
    __syncwarp();
    const float kInf = __int_as_float(0x7f800000), kNaN = __int_as_float(0x7fffffff);

    for (uint32_t base = s0; base < s1; base += 32) {
        const uint32_t ni = s1 - base < 32u ? s1 - base : 32u;
        const bool act = (uint32_t)lane < ni;
        const uint32_t me = base + lane;
        if (act) {
            // an atom whose offset is not exact carries NaN in z and w: its
            // pairs fail every FP32 test (w is the flag the FP32 tests read)
            float4 o = A.o0[me];
            if (o.w != 0.0f) o.z = o.w = kNaN;
            S.oi[lane] = o;
            S.origi[lane] = A.orig[me];
        }
        // this atom's own candidate index (it is a candidate of its own cell)
        const uint32_t self_t = act ? S.cpre[home] + (me - S.cj0[home]) : 0xffffffffu;
        __syncwarp();
        int cnt = 0;  // list length of atom `me`
        int c = 0;    // neighbour cell of this lane's candidate
        for (uint32_t tb = 0; tb < T; tb += 32) {
            const uint32_t t = tb + lane;
            const bool have = t < T;
            uint32_t j = 0xffffffffu, origj = 0;
            float px = 0.f, py = 0.f, pz = 0.f;
            bool pfj = false;
            if (have) {
                while (S.cpre[c + 1] <= t) ++c;
                j = S.cj0[c] + (t - S.cpre[c]);
                const float4 oj = A.o0[j];
                const float4 shj = S.csh[c];
                // the candidate seen from the cell: offset + image shift
                px = oj.x + shj.x;
                py = oj.y + shj.y;
                pz = oj.z + shj.z;
                pfj = uniform_rns && oj.w == 0.0f;
                if (A.half) origj = A.orig[j];
                S.cand[lane] = j | S.ccode[c];
            }
            __syncwarp();
            // row ii of the chunk's accept matrix lands in lane ii; pairs
            // within 1e-5 of rns (or of atoms whose offsets are not exact)
            // are marked in a second row and settled in FP64 below
            unsigned mine = 0, mine_x = 0;
            bool exact = A.half;
            if (!A.half) {
                // One ballot per atom: the candidate's coordinates are +inf
                // without a candidate and NaN when the prefilter cannot
                // decide its pairs, so neither is ever accepted here; the
                // atom's own slot is cleared after the loop. A pair that the
                // prefilter cannot settle (band, NaN) sends the whole chunk
                // to the loop below, whose rows are therefore the same.
                const float qx = !have ? kInf : pfj ? px : kNaN;
                bool band = false;
#pragma unroll 2
                for (uint32_t ii = 0; ii < ni; ++ii) {
                    const float4 oi = S.oi[ii];
                    const float dx = oi.x - qx, dy = oi.y - py, dz = oi.z - pz;
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const bool sure = d2 < lo2;
                    const unsigned m = __ballot_sync(full, sure);
                    band |= !sure && !(d2 > hi2);
                    if ((uint32_t)lane == ii) mine = m;
                }
                if (self_t - tb < 32u) mine &= ~(1u << (self_t - tb));
                exact = __any_sync(full, band);
            }
            if (exact) {
                mine = 0;
#pragma unroll 2
                for (uint32_t ii = 0; ii < ni; ++ii) {
                    const float4 oi = S.oi[ii];
                    const float dx = oi.x - px, dy = oi.y - py, dz = oi.z - pz;
                    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                    const bool pf = pfj && oi.w == 0.0f;
                    const bool ok = have && j != base + ii && !(A.half && origj < S.origi[ii]);
                    const unsigned m = __ballot_sync(full, ok && pf && d2 < lo2);
                    const unsigned mx = __ballot_sync(full, ok && !(pf && (d2 < lo2 || d2 > hi2)));
                    if ((uint32_t)lane == ii) {
                        mine = m;
                        mine_x = mx;
                    }
                }
            }
            while (mine_x) {
                const int b = __ffs(mine_x) - 1;
                mine_x &= mine_x - 1u;
                const uint32_t jb = S.cand[b] & kJMask;
                if (are_neibs_exact(g, A.rx[me], A.ry[me], A.rz[me], A.rns[me], A.rx[jb], A.ry[jb], A.rz[jb],
                                    A.rns[jb], edge))
                    mine |= 1u << b;
            }
            // append this atom's accepted candidates in candidate order
            while (mine) {
                const int b = __ffs(mine) - 1;
                mine &= mine - 1u;
                if (cnt < A.K) A.nbr[nidx(cnt, me, A.np)] = S.cand[b];
                ++cnt;
            }
            __syncwarp();
        }
        if (act) {
            const int padded = (cnt + 3) & ~3;
            for (int k = cnt; k < padded && k < A.K; ++k) A.nbr[nidx(k, me, A.np)] = me | kSelfCode;
            A.ncnt[me] = padded < A.K ? padded : A.K;
            if (cnt > A.K) {
                atomicOr(&A.st->flags, FLAG_OVERFLOW);
                atomicOr(&A.st->build_flags, FLAG_OVERFLOW);
            }
            A.r0x[me] = A.rx[me];
            A.r0y[me] = A.ry[me];
            A.r0z[me] = A.rz[me];
            A.saved_rcut[me] = A.rcut[me];
            A.saved_rns[me] = A.rns[me];
            A.saved_uid[me] = A.uid[me];
        }
        // the longest list, one atomic per warp
        const unsigned wmax = __reduce_max_sync(full, act ? (unsigned)cnt : 0u);
        if (lane == 0) atomicMax(&A.st->max_count, wmax);
        __syncwarp();
    }
}

}  // namespace mdg

struct mdg_system;

namespace mdg {
// Host-side argument builders of a system's rebuild (nlist.cu).
GatherAll gather_sets(const mdg_system* sys);
NbArgs nb_args(const mdg_system* sys);
DomainDev domain_of(const mdg_system* sys);
}  // namespace mdg
