// mdg_internal.cuh — device data layout and shared helpers of libmdg.
//
// Layout in HBM (one system, atoms in cell-sorted "slot" order):
//   FP64 SoA  rx ry rz | vx vy vz | fx fy fz (FP64 forces) | m rcut rns
//             Rx Ry Rz (FP64 centre of the atom's cell at the last rebuild)
//             Ep Em nc, V[9][n] (per-atom measurement outputs)
//   FP32      f32[3][n] (mixed forces), o0 float4 (FP32 offsets from the
//             cell centre at the rebuild, read by the list build)
//   fixed     pos32 int4 {x,y,z offset from the cell centre in units of
//             cs / 2^29 per axis, w = bits of the FP32 EAM F'(rho)}
//   ints      orig (slot -> caller index), uid, kind (u16), tag (u16),
//             cell (packed local cell coordinates)
//   list      ELL: nbr[k * np + i] (k < K), ncnt[i]; entry = j | image << 25
//             where image packs the cell offset of j's periodic image as
//             2 bits per axis (value + 1).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mdg.h"

namespace mdg {

constexpr int kJBits = 25;
constexpr uint32_t kJMask = (1u << kJBits) - 1u;
constexpr uint32_t kMaxAtoms = (1u << kJBits);
constexpr int kMaxKinds = 4;
constexpr int kBlock = 256;

enum : uint32_t {
    FLAG_RANGE = 1u,      // atom outside the local grid (clamped)
    FLAG_OVERFLOW = 2u,   // neighbour count above capacity
    FLAG_TABLE = 4u,      // EAM table range / extrapolation branch taken
    FLAG_NONFINITE = 8u,  // non-finite force
    FLAG_IMAGE = 16u,     // periodic image offset outside {-1,0,1}
};

// Linked-cell grid of the last rebuild (mdcraft/neibs/grid.cxx:43-95),
// computed on the device from the atoms' bounds.
struct GridParams {
    int dom_n[3];      // domain_num_cells
    int offset[3];     // grid_offset
    int num[3];        // num_cells (local grid)
    int bricks[3];     // ceil(num / 4)
    int dim;
    int periodic[3];
    int small_box;     // some periodic axis has <= 2 cells, or a local grid short of it: the per-atom
                       // build with per-pair minimum-image codes (FP32 prefilter on a whole grid,
                       // the exact FP64 test for every candidate on a local grid short of the box)
    int ncells;
    int nbins;         // 64 * bricks product
    int empty;
    double cs[3];      // cell_sizes
    double bmin[3];    // domain
    double bmax[3];
    double size[3];
    double gmin[3];    // bmin + cs * offset (local grid origin)
    double max_rns;
    float csf[3];
    float Lf[3];
    double inv_u[3];   // 2^29 / cs: FP64 offset -> fixed-point units (pos32)
    double inv_cs[3];  // 1 / cs, for the cell of a position (floor_div)
};

// Fixed-point cell offsets of the mixed form. An offset from the atom's cell
// centre is stored as an integer number of units u = cs / 2^29 per axis
// (range +-4 cells), so the pair vector r_j - r_i = (o_j - o_i) + image
// cells * 2^29 is an exact integer: the only rounding is its conversion to
// FP32, and pairs related by inversion symmetry get exactly opposite vectors.
// (Differences of independently rounded FP32 offsets break that symmetry:
// on a perfect lattice they left forces that should cancel at ~1e-5 of the
// RMS force.)
constexpr int kOffBits = 29;
constexpr double kOffUnits = 536870912.0;  // 2^29

__device__ __forceinline__ int off_encode(double d, double inv_u) { return __double2int_rn(d * inv_u); }

// Bricked-Morton bin key of a local cell: 4x4x4 bricks in x-fastest order,
// Morton order inside a brick.
__host__ __device__ inline int bin_key(const GridParams& g, int cx, int cy, int cz) {
    int bx = cx >> 2, by = cy >> 2, bz = cz >> 2;
    int lx = cx & 3, ly = cy & 3, lz = cz & 3;
    int m = (lx & 1) | ((ly & 1) << 1) | ((lz & 1) << 2) | ((lx & 2) << 2) |
            ((ly & 2) << 3) | ((lz & 2) << 4);
    return ((bz * g.bricks[1] + by) * g.bricks[0] + bx) * 64 + m;
}

__host__ __device__ inline uint32_t pack_cell(int cx, int cy, int cz) {
    return (uint32_t)cx | ((uint32_t)cy << 10) | ((uint32_t)cz << 20);
}
__host__ __device__ inline void unpack_cell(uint32_t p, int& cx, int& cy, int& cz) {
    cx = (int)(p & 1023u);
    cy = (int)((p >> 10) & 1023u);
    cz = (int)((p >> 20) & 1023u);
}

// Position of list entry k of atom (slot) i: entries are stored in groups of
// four per atom ("ELL4"), so a thread reads four neighbours with one 16-byte
// load and a warp reads 512 contiguous bytes per group. Lists are padded to
// a multiple of four with self entries (r = 0, excluded by every force
// kernel's r^2 >= 1e-15 test).
__host__ __device__ inline size_t nidx(int k, size_t i, size_t np) {
    return (((size_t)(k >> 2) * np + i) << 2) + (size_t)(k & 3);
}
constexpr uint32_t kSelfCode = 0x15u << kJBits;  // image (0,0,0)

// Image offset encoded in a list entry (2 bits per axis, value+1), in
// fixed-point offset units (-2^29, 0, 2^29; modulo 2^32).
__device__ inline uint32_t image_units(uint32_t e, int axis) {
    uint32_t b = (e >> (kJBits + 2 * axis)) & 3u;  // 0, 1, 2 for -1, 0, +1 cells
    return (b - 1u) << kOffBits;
}

// Potential types: LJsCut and the tabulated Pair are the reference's
// potential::type::pair (one force stage), EAM its potential::type::eam.
enum : int { POT_NONE = 0, POT_LJCUT = 1, POT_EAM = 2, POT_TAB = 3, POT_LJS = 4 };

// Per-kind-pair potential parameters handed to the force kernels by value.
// Every table pointer is valid (a zero table stands in where a potential
// has none), so a load the compiler issues ahead of its condition stays
// in bounds.
struct PotParams {
    int type;          // POT_*
    double R2cut;
    float r2cut_f;
    // LJsCut (LJs-cut.cxx:8-20)
    double a, s6, lj1, lj2, factor;
    float lj1_f, lj2_f, mhf_f;  // mhf = -0.5 * factor
    // LJs (LJs.cxx:7-29), after its constructor's rescaling
    double ljs_rVr1, ljs_rVr2, ljs_aLJ, ljs_bLJ, ljs_aLJ3, ljs_bLJ2, ljs_aVr, ljs_aVr2;
    float ljs_rVr1_f, ljs_rVr2_f, ljs_aLJ_f, ljs_bLJ_f, ljs_aVr2_f;
    // EAM tables, FP64 values + knot slopes with one padding element
    int Nr1, Nrh1;
    double dr, drh, dr1, drh1;
    const double* Rho;
    const double* dRho;
    const double* Vpar;
    const double* dVpar;
    const double* Femb;
    const double* dFemb;
    // FP32 cubic coefficients per interval (u-form, u in [0,1))
    const float4* rho_c;
    const float4* v_c;
    const float4* f_c;
    const float4* rv_c;  // force rows: W(u) = V'r - V, then D(u) = rho' (2 float4 per interval)
    float inv_dr_f, inv_drh_f, dr1_f, drh_f;
};

struct PotSet {
    int nkinds;       // 1 for Single (atom kinds ignored)
    int multi;
    int any_eam;
    int periodic;     // boundary::Periodic
    int any_lj, any_tab, any_ljs;
    PotParams p[kMaxKinds][kMaxKinds];
};

// Rows of the zero table every table-less PotParams points at: enough for
// the widest unconditional read (an interleaved rho/V row at interval 0,
// FP64 knots 0 and 1).
constexpr int kZeroRows = 8;

// thermostat::Langevin terms (mdcraft/solver/thermostat/langevin.cxx),
// applied in order after the force stage; sigma = sqrt(2 beta Kb T / dt).
constexpr int kMaxThermo = 8;
struct LangevinTerm {
    double beta, sigma;
    double heat[3], U[3];
    double xmin, xmax;
    unsigned long long seed;
};
struct ThermoDev {
    int n;
    int pad;
    LangevinTerm t[kMaxThermo];
};

// Exact FP64 arithmetic without contraction, for bit-for-bit parity with
// the reference's host arithmetic.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ double sq3_exact(double x, double y, double z) {
    return dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
}

// Domain::shortest (mdcraft/lattice/domain.cxx:59-66), one axis.
__device__ __forceinline__ double shortest1(double v, double L, int periodic) {
    if (!periodic) return v;
    v = fabs(dadd(v, L)) < fabs(v) ? dadd(v, L) : v;
    v = fabs(dsub(v, L)) < fabs(v) ? dsub(v, L) : v;
    return v;
}

// Device-side status words of one system.
struct DevStatus {
    uint32_t flags;         // FLAG_* accumulated until read by mdg_system_flags
    uint32_t need_rebuild;  // rebuild test of the current step
    uint32_t max_count;     // longest list of the last build
    uint32_t nonuniform;    // some atom's rns differs from atom 0's
    uint32_t build_flags;   // FLAG_* raised by the current rebuild
    uint32_t pad[2];
    uint32_t therm_calls;   // thermostat applications so far (Philox counter word)
    uint32_t need_next;     // rebuild test of the next step's positions, from a force pass
                            // that ran the next step's first half-kick and drift
};

}  // namespace mdg
