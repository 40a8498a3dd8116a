// forces_dev.cuh — per-atom bodies of the mixed-precision force stages,
// shared by the per-stage kernels (forces.cu) and the fused per-system loop
// (solo.cu), so both give the same forces bit for bit.
//
// LJsCut::compute / EAM::charge and forces (mdcraft/solver/potential/
// LJs-cut.cxx:22-131, EAM.cxx:141-601) in FP32 pair arithmetic on pair
// vectors taken exactly from fixed-point cell-centred offsets, with
// compensated per-atom sums.
#pragma once

#include <cuda_runtime.h>

#include "mdg_internal.cuh"

namespace mdg {

// A group of four list entries: streamed once per pass, so kept out of L1
// (the gathers of neighbour records and table rows keep it).
__device__ __forceinline__ uint4 ldg_list(const uint4* p) {
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}


struct FArgs {
    int n, np;
    const double *rx, *ry, *rz, *rns;
    const uint32_t *nbr, *ncnt;
    const uint16_t *kind, *tag;
    const uint8_t* bc;
    double L[3];
    int periodic[3];
    float uf[3];  // length of one fixed-point offset unit per axis, cs / 2^29 in FP32
    // outputs / intermediate
    double *fx, *fy, *fz;
    float *gx, *gy, *gz;  // mixed forces
    double* nc;
    double* Fp64;
    float* Fp32;
    const int4* pos32;  // fixed-point offsets (mdg_internal.cuh)
    int4* pos32b;       // the same offsets with w = bits of the FP32 F'(rho) (EAM)
    uint32_t* cutbits;  // null, or the density pass's FP64 decisions of band pairs (mdg_system::cutbits)
    double *Ep, *Em;
    double* V[9];
    DevStatus* st;
    // second half-kick fused into the force pass (mixed form): v += g * hdt / m
    const double* m;
    double *vx, *vy, *vz;
    float kick_hdt;  // 0.5f * (float)dt
};

// Stores the atom's FP32 force and, with KICK, applies the second half-kick
// exactly as kick_mixed_one does (same FP32 product, same rounding).
template <bool KICK>
__device__ __forceinline__ void store_force(const FArgs& A, int i, float fx, float fy, float fz) {
    A.gx[i] = fx;
    A.gy[i] = fy;
    A.gz[i] = fz;
    if (KICK) {
        const float hm = A.kick_hdt * __frcp_rn((float)A.m[i]);
        A.vx[i] += (double)(fx * hm);
        A.vy[i] += (double)(fy * hm);
        A.vz[i] += (double)(fz * hm);
    }
}

// ---------------------------------------------------------------------------
// mixed precision
// ---------------------------------------------------------------------------
struct Kahan3 {
    float s[3] = {0.f, 0.f, 0.f};
    float c[3] = {0.f, 0.f, 0.f};
    __device__ __forceinline__ void add(int k, float v) {
        float y = v - c[k];
        float t = s[k] + y;
        c[k] = (t - s[k]) - y;
        s[k] = t;
    }
};

__device__ __forceinline__ float ksum_add(float& s, float& c, float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
    return s;
}

// Pair vector r_j - r_i of a list entry from the fixed-point cell-centred
// offsets: an exact integer difference (modulo 2^32; the true value is
// within +-2^31 units), one rounding to FP32, one scaling by the unit.
__device__ __forceinline__ void pair_vec32(uint32_t e, const int4& pi, const int4& pj, const float uf[3],
                                           float& dx, float& dy, float& dz) {
    dx = __int2float_rn((int)((uint32_t)pj.x - (uint32_t)pi.x + image_units(e, 0))) * uf[0];
    dy = __int2float_rn((int)((uint32_t)pj.y - (uint32_t)pi.y + image_units(e, 1))) * uf[1];
    dz = __int2float_rn((int)((uint32_t)pj.z - (uint32_t)pi.z + image_units(e, 2))) * uf[2];
}

// 1/sqrt(x) for x > 0: the hardware estimate refined by one Newton step, so
// r = x * rinv and 1/r are nearly correctly rounded (pair forces near an
// equilibrium lattice cancel, which magnifies their relative errors).
__device__ __forceinline__ float rsqrt_nr(float x) {
    const float y = rsqrtf(x);
    return y * fmaf(-0.5f * x * y, y, 1.5f);
}

// Both force rows (W, D) of one interval: 32 bytes, one 256-bit load
// (measured: EAM Cu 1M force pass 0.208 ms, against 0.216 ms with separate
// tables and 0.245 ms with two 128-bit loads of the interleaved rows).
__device__ __forceinline__ void load_rv(const float4* rv, int nn, float4& cw, float4& cd) {
    const float4* p = rv + 2 * nn;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(cw.x), "=f"(cw.y), "=f"(cw.z), "=f"(cw.w), "=f"(cd.x), "=f"(cd.y), "=f"(cd.z), "=f"(cd.w)
        : "l"(p));
}

__device__ __forceinline__ float cubic(const float4 c, float u) {
    return fmaf(u, fmaf(u, fmaf(u, c.w, c.z), c.y), c.x);
}
__device__ __forceinline__ float dcubic(const float4 c, float u) {
    return fmaf(u, fmaf(u, 3.0f * c.w, 2.0f * c.z), c.y);
}

// Pair entries whose image crossed a periodic face contribute only with
// the Periodic boundary (without it the reference's raw distance is beyond
// the cutoff); bit 31 marks them.
constexpr uint32_t kWrapBit = 1u << 31;

// Cutoff membership of a pair. The FP32 r^2 decides unless it lies within
// 1e-5 (relative) of rc^2; those rare pairs are decided on the FP64
// positions, so the mixed form cuts exactly the pairs the FP64 form cuts
// (the potentials are discontinuous at rc, so a flipped pair would change
// forces by a whole pair term).
__device__ __forceinline__ bool cut_in(const FArgs& A, int i, uint32_t j, float r2, float r2c, double R2cut) {
    if (r2 < 1e-15f) return false;
    float band = 1e-5f * r2c;
    if (r2 < r2c - band) return true;
    if (r2 > r2c + band) return false;
    double dx = shortest1(A.rx[j] - A.rx[i], A.L[0], A.periodic[0]);
    double dy = shortest1(A.ry[j] - A.ry[i], A.L[1], A.periodic[1]);
    double dz = shortest1(A.rz[j] - A.rz[i], A.L[2], A.periodic[2]);
    return dx * dx + dy * dy + dz * dz <= R2cut;
}

// Cutoff membership from the FP32 r^2, with the rare pairs inside the
// 1e-5 band around rc^2 (and entries that crossed a periodic face when the
// solver has no Periodic boundary) settled exactly.
__device__ __forceinline__ bool pair_in(const FArgs& A, int i, uint32_t e, float r2, float r2c, double R2c,
                                        bool per) {
    bool in = r2 >= 1e-15f && r2 <= r2c;
    if (fabsf(r2 - r2c) <= 1e-5f * r2c) in = cut_in(A, i, e & kJMask, r2, r2c, R2c);
    return in && (per || !(e & kWrapBit));
}

// pair_in for the density pass of a step whose force pass moves atoms: the
// FP64 decisions of the band pairs (entry k of atom i) are also collected in
// *bits, one bit per entry, and *band notes that the word has one.
__device__ __forceinline__ bool pair_in_rec(const FArgs& A, int i, uint32_t e, float r2, float r2c, double R2c,
                                            bool per, int k, uint32_t* bits, bool* band) {
    bool in = r2 >= 1e-15f && r2 <= r2c;
    if (fabsf(r2 - r2c) <= 1e-5f * r2c) {
        in = cut_in(A, i, e & kJMask, r2, r2c, R2c);
        *bits |= (uint32_t)in << (k & 31);
        *band = true;
    }
    return in && (per || !(e & kWrapBit));
}

// pair_in for such a force pass: a band pair takes the density pass's FP64
// decision (the same FP32 r^2 puts it in the band there), so the pass reads
// no neighbour's FP64 position.
__device__ __forceinline__ bool pair_in_bits(const FArgs& A, int i, uint32_t e, float r2, float r2c, bool per,
                                             int k) {
    bool in = r2 >= 1e-15f && r2 <= r2c;
    if (fabsf(r2 - r2c) <= 1e-5f * r2c) in = (__ldg(A.cutbits + (size_t)(k >> 5) * A.np + i) >> (k & 31)) & 1u;
    return in && (per || !(e & kWrapBit));
}

// The pair loops below read four list entries with one 16-byte load, then
// the four neighbour records, so the loads of a group overlap; the four
// contributions are summed in FP32 and the group sum enters a Kahan sum.

template <bool MULTI>
__device__ __forceinline__ bool lj_mixed_force(const FArgs& A, const PotSet* __restrict__ ps, int i, float& out_x,
                                             float& out_y, float& out_z) {
    if (A.tag[i] == 0) return false;
    const int4 pi = A.pos32[i];
    const int ng = A.ncnt[i] >> 2;
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const bool per = ps->periodic;
    const float uf[3] = {A.uf[0], A.uf[1], A.uf[2]};
    const PotParams& P0 = ps->p[ki][0];
    float r2c = P0.r2cut_f, l1 = P0.lj1_f, l2 = P0.lj2_f, mh = P0.mhf_f;
    double R2c = P0.R2cut;
    Kahan3 acc;
    const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
    uint4 e4n = ng > 0 ? ldg_list(row) : make_uint4(0, 0, 0, 0);
    for (int g = 0; g < ng; ++g) {
        // the next group's entries are requested before this group's work
        const uint4 e4 = e4n;
        if (g + 1 < ng) e4n = ldg_list(row + (size_t)(g + 1) * A.np);
        const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
        int4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32 + (e[q] & kJMask));
        float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (MULTI) {
                const PotParams& P = ps->p[ki][pj[q].w & 3];
                r2c = P.r2cut_f; l1 = P.lj1_f; l2 = P.lj2_f; mh = P.mhf_f; R2c = P.R2cut;
            }
            float dx, dy, dz;
            pair_vec32(e[q], pi, pj[q], uf, dx, dy, dz);
            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool in = pair_in(A, i, e[q], r2, r2c, R2c, per);
            float r2inv = __fdividef(1.0f, fmaxf(r2, 1e-12f));
            float r6inv = r2inv * r2inv * r2inv;
            float pref = in ? mh * fmaf(l1, r6inv, -l2) * r6inv * r2inv : 0.f;
            fx = fmaf(dx, pref, fx);
            fy = fmaf(dy, pref, fy);
            fz = fmaf(dz, pref, fz);
        }
        acc.add(0, fx);
        acc.add(1, fy);
        acc.add(2, fz);
    }
    out_x = acc.s[0];
    out_y = acc.s[1];
    out_z = acc.s[2];
    return true;
}

template <bool MULTI, bool KICK = false>
__device__ __forceinline__ void lj_mixed_one(const FArgs& A, const PotSet* __restrict__ ps, int i) {
    float fx, fy, fz;
    if (lj_mixed_force<MULTI>(A, ps, i, fx, fy, fz)) store_force<KICK>(A, i, fx, fy, fz);
}

// Force / r of a tabulated Pair term (pair.cxx:316-346) in FP32 from the
// cubic coefficients of its r*phi table: d(r phi)/dr * r - r phi, over r^3.
__device__ __forceinline__ float tab_ff32(const PotParams& P, float r2, bool& in) {
    const float rinv = rsqrt_nr(fmaxf(r2, 1e-12f));
    const float r = r2 * rinv;
    const float t = r * P.inv_dr_f;
    int nn = (int)t;
    in = in && nn < P.Nr1;
    nn = in ? nn : 0;
    const float u = t - (float)nn;
    const float4 cv = __ldg(P.v_c + nn);
    const float V = cubic(cv, u);
    const float dV = dcubic(cv, u) * P.inv_dr_f;
    return (dV * r - V) * (rinv * rinv) * rinv;
}

__device__ __forceinline__ float lj_ff32(const PotParams& P, float r2) {
    const float r2inv = __fdividef(1.0f, fmaxf(r2, 1e-12f));
    const float r6inv = r2inv * r2inv * r2inv;
    return P.mhf_f * fmaf(P.lj1_f, r6inv, -P.lj2_f) * r6inv * r2inv;
}

// Force / r of an LJs pair (LJs.cxx:153-166) in FP32.
__device__ __forceinline__ float ljs_ff32(const PotParams& P, float r2) {
    const float XX = fmaf(P.ljs_rVr1_f, r2, -1.2599210498948732f);
    const float FV = P.ljs_rVr2_f * __fdividef(1.0f, fmaxf(r2, 1e-12f));
    const float Ur = FV * FV * FV;
    return P.ljs_aVr2_f * fmaf(Ur * (Ur - 0.5f), FV, fmaf(P.ljs_bLJ_f, XX, P.ljs_aLJ_f) * XX);
}

// Force / r of an analytic pair potential by type (LJsCut or LJs).
__device__ __forceinline__ float analytic_ff32(const PotParams& P, float r2) {
    return P.type == POT_LJS ? ljs_ff32(P, r2) : lj_ff32(P, r2);
}

// Pair-type forces (no EAM term) beyond the plain LJsCut kernel: FORM 3 =
// every pair a tabulated Pair, 4 = every pair LJs, 0 = chosen per kind pair
// among LJsCut, Pair and LJs.
template <bool MULTI, int FORM>
__device__ __forceinline__ bool pair_mixed_force(const FArgs& A, const PotSet* __restrict__ ps, int i, float& out_x,
                                             float& out_y, float& out_z) {
    if (A.tag[i] == 0) return false;
    const int4 pi = A.pos32[i];
    const int ng = A.ncnt[i] >> 2;
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const bool per = ps->periodic;
    const float uf[3] = {A.uf[0], A.uf[1], A.uf[2]};
    Kahan3 acc;
    const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
    uint4 e4n = ng > 0 ? ldg_list(row) : make_uint4(0, 0, 0, 0);
    for (int g = 0; g < ng; ++g) {
        const uint4 e4 = e4n;
        if (g + 1 < ng) e4n = ldg_list(row + (size_t)(g + 1) * A.np);
        const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
        int4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32 + (e[q] & kJMask));
        float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const PotParams& P = ps->p[ki][MULTI ? (pj[q].w & 3) : 0];
            float dx, dy, dz;
            pair_vec32(e[q], pi, pj[q], uf, dx, dy, dz);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool in = pair_in(A, i, e[q], r2, P.r2cut_f, P.R2cut, per);
            float FF;
            if (FORM == 3 || (FORM == 0 && P.type == POT_TAB)) {
                FF = tab_ff32(P, r2, in);
            } else if (FORM == 4) {
                FF = ljs_ff32(P, r2);
            } else {
                in = in && (P.type == POT_LJCUT || P.type == POT_LJS);
                FF = analytic_ff32(P, r2);
            }
            FF = in ? FF : 0.f;
            fx = fmaf(dx, FF, fx);
            fy = fmaf(dy, FF, fy);
            fz = fmaf(dz, FF, fz);
        }
        acc.add(0, fx);
        acc.add(1, fy);
        acc.add(2, fz);
    }
    out_x = acc.s[0];
    out_y = acc.s[1];
    out_z = acc.s[2];
    return true;
}

template <bool MULTI, int FORM, bool KICK = false>
__device__ __forceinline__ void pair_mixed_one(const FArgs& A, const PotSet* __restrict__ ps, int i) {
    float fx, fy, fz;
    if (pair_mixed_force<MULTI, FORM>(A, ps, i, fx, fy, fz)) store_force<KICK>(A, i, fx, fy, fz);
}

__device__ __forceinline__ void embed32(const PotParams& P, float rho, float* F, float* dF,
                                        DevStatus* st) {
    float t = rho * P.inv_drh_f;
    if (!(t >= 0.0f) || t >= (float)(P.Nrh1 - 1)) {
        atomicOr(&st->flags, FLAG_TABLE);
        t = fminf(fmaxf(t, 0.0f), (float)(P.Nrh1 - 1) - 1e-3f);
    }
    int nn = (int)t;
    float u = t - (float)nn;
    float4 c = __ldg(P.f_c + nn);
    *F = cubic(c, u);
    *dF = dcubic(c, u) * P.inv_drh_f;
}

// REC: also record the FP64 decisions of the band pairs in A.cutbits, for a
// force pass that moves atoms (pair_in_rec).
template <bool MULTI, bool REC = false>
__device__ __forceinline__ void density_mixed_one(const FArgs& A, const PotSet* __restrict__ ps, int i) {
    const int4 pi = A.pos32[i];
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const float uf[3] = {A.uf[0], A.uf[1], A.uf[2]};
    const bool per = ps->periodic;
    float s = 0.f, c = 0.f;
    if (A.tag[i] != 0) {
        const int ng = A.ncnt[i] >> 2;
        const PotParams* P = &ps->p[ki][0];
        float r2c = P->r2cut_f, idr = P->inv_dr_f;
        double R2c = P->R2cut;
        int Nr1 = P->Nr1;
        const float4* tab = P->rho_c;
        const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
        uint4 e4n = ng > 0 ? ldg_list(row) : make_uint4(0, 0, 0, 0);
        uint32_t bits = 0;   // FP64 cut decisions of this word's band entries, for A.cutbits
        bool band = false;  // the word has a band entry
        for (int g = 0; g < ng; ++g) {
            // the next group's entries are requested before this group's work
            const uint4 e4 = e4n;
            if (g + 1 < ng) e4n = ldg_list(row + (size_t)(g + 1) * A.np);
            const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
            int4 pj[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32 + (e[q] & kJMask));
            float part = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                bool eam = true;
                if (MULTI) {
                    P = &ps->p[ki][pj[q].w & 3];  // the partner's kind rides in its offsets' w
                    r2c = P->r2cut_f; idr = P->inv_dr_f; Nr1 = P->Nr1; tab = P->rho_c; R2c = P->R2cut;
                    eam = P->type == 2;
                }
                float dx, dy, dz;
                pair_vec32(e[q], pi, pj[q], uf, dx, dy, dz);
                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                bool in;
                if (REC)  // every pair's band decision, whatever its potential
                    in = pair_in_rec(A, i, e[q], r2, r2c, R2c, per, 4 * g + q, &bits, &band) && eam;
                else
                    in = eam && pair_in(A, i, e[q], r2, r2c, R2c, per);
                float t = r2 * rsqrt_nr(fmaxf(r2, 1e-12f)) * idr;
                int nn = (int)t;
                in = in && nn < Nr1;
                nn = in ? nn : 0;
                float u = t - (float)nn;
                float v = in ? cubic(__ldg(tab + nn), u) : 0.f;
                part += v;
            }
            ksum_add(s, c, part);
            if (REC && ((g & 7) == 7 || g + 1 == ng)) {
                if (band) A.cutbits[(size_t)(g >> 3) * A.np + i] = bits;
                bits = 0;
                band = false;
            }
        }
    }
    float rho = s;
    // the atom's density as the reference's charge stage leaves it (FP32 sum here)
    if (A.tag[i] != 0) A.nc[i] = (double)rho;
    float Fp0 = 0.f;
    for (int b = 0; b < ps->nkinds; ++b) {
        const PotParams& P = ps->p[ki][b];
        float F = 0.f, dF = 0.f;
        if (P.type == 2) embed32(P, rho, &F, &dF, A.st);
        if (b == 0) Fp0 = dF;
        if (MULTI) A.Fp32[(size_t)b * A.np + i] = dF;
    }
    // Multi: the two lowest mantissa bits of F' (relative 2^-22, below the
    // FP32 sums' own rounding) carry the atom's kind for the force pass
    const int w = MULTI ? ((__float_as_int(Fp0) & ~3) | ki) : __float_as_int(Fp0);
    A.pos32b[i] = make_int4(pi.x, pi.y, pi.z, w);
}

// BITS: a pair in the 1e-5 band around the cutoff takes the density pass's
// FP64 decision (A.cutbits) rather than testing the FP64 positions itself;
// the force pass then reads no FP64 position of a neighbour (what a force
// pass that moves its atoms needs).
template <bool MULTI, bool BITS = false>
__device__ __forceinline__ bool eam_mixed_force(const FArgs& A, const PotSet* __restrict__ ps, int i, float& out_x,
                                             float& out_y, float& out_z) {
    if (A.tag[i] == 0) return false;
    const int4 pi = A.pos32b[i];
    const int ng = A.ncnt[i] >> 2;
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const float uf[3] = {A.uf[0], A.uf[1], A.uf[2]};
    const bool per = ps->periodic;
    const PotParams* P = &ps->p[ki][0];
    float r2c = P->r2cut_f, idr = P->inv_dr_f;
    double R2c = P->R2cut;
    int Nr1 = P->Nr1;
    const float4* rv = P->rv_c;
    Kahan3 acc;
    // Multi: F' of atom i for the kinds 1..3 of its partners, read once (the
    // density pass's Fp32 rows; kind 0's is the record's w, with the atom's
    // kind in its two lowest bits)
    float fpi1 = 0.f, fpi2 = 0.f, fpi3 = 0.f;
    if (MULTI) {
        const int nk = ps->nkinds;
        if (nk > 1) fpi1 = A.Fp32[A.np + i];
        if (nk > 2) fpi2 = A.Fp32[2 * (size_t)A.np + i];
        if (nk > 3) fpi3 = A.Fp32[3 * (size_t)A.np + i];
    }
    const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
    uint4 e4n = ng > 0 ? ldg_list(row) : make_uint4(0, 0, 0, 0);
    for (int g = 0; g < ng; ++g) {
        // the next group's entries are requested before this group's work
        const uint4 e4 = e4n;
        if (g + 1 < ng) e4n = ldg_list(row + (size_t)(g + 1) * A.np);
        const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
        int4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32b + (e[q] & kJMask));
        float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float Fpi = __int_as_float(MULTI ? pi.w & ~3 : pi.w), Fpj = __int_as_float(MULTI ? pj[q].w & ~3 : pj[q].w);
            bool eam = true, lj = false;
            if (MULTI) {
                uint32_t j = e[q] & kJMask;
                const int kj = pj[q].w & 3;
                P = &ps->p[ki][kj];
                // a tabulated Pair has zero rho rows: the EAM arithmetic
                // below reduces to its pair term exactly
                eam = P->type == POT_EAM || P->type == POT_TAB;
                lj = P->type == POT_LJCUT || P->type == POT_LJS;
                r2c = P->r2cut_f; idr = P->inv_dr_f; Nr1 = P->Nr1; rv = P->rv_c; R2c = P->R2cut;
                // j's F' for i's kind (kind 0's is in j's record)
                if (ki != 0) Fpj = A.Fp32[(size_t)ki * A.np + j];
                Fpi = kj == 0 ? Fpi : kj == 1 ? fpi1 : kj == 2 ? fpi2 : fpi3;
            }
            float dx, dy, dz;
            pair_vec32(e[q], pi, pj[q], uf, dx, dy, dz);
            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool in;
            if (BITS) in = (eam || lj) && pair_in_bits(A, i, e[q], r2, r2c, per, 4 * g + q);
            else in = (eam || lj) && pair_in(A, i, e[q], r2, r2c, R2c, per);
            // one reciprocal square root gives both r and 1/r
            float rinv = rsqrt_nr(fmaxf(r2, 1e-12f));
            float r = r2 * rinv;
            float t = r * idr;
            int nn = (int)t;
            in = in && (lj || nn < Nr1);
            nn = in && !lj ? nn : 0;
            float u = t - (float)nn;
            float4 cw, cd;
            load_rv(rv, nn, cw, cd);
            // W = V'r - V and D = rho' on the interval (force_rows)
            const float W = cubic(cw, u);
            const float D = fmaf(u, fmaf(u, cd.z, cd.y), cd.x);
            float FF = fmaf(Fpi + Fpj, D, W * (rinv * rinv)) * rinv;
            if (MULTI && lj) FF = analytic_ff32(*P, r2);
            FF = in ? FF : 0.f;
            fx = fmaf(FF, dx, fx);
            fy = fmaf(FF, dy, fy);
            fz = fmaf(FF, dz, fz);
        }
        acc.add(0, fx);
        acc.add(1, fy);
        acc.add(2, fz);
    }
    out_x = acc.s[0];
    out_y = acc.s[1];
    out_z = acc.s[2];
    return true;
}

template <bool MULTI, bool KICK = false>
__device__ __forceinline__ void eam_mixed_one(const FArgs& A, const PotSet* __restrict__ ps, int i) {
    float fx, fy, fz;
    if (eam_mixed_force<MULTI>(A, ps, i, fx, fy, fz)) store_force<KICK>(A, i, fx, fy, fz);
}

}  // namespace mdg

struct mdg_system;

namespace mdg {
// Argument block of a system's force stages (forces.cu).
FArgs force_args(mdg_system* sys);
}  // namespace mdg
