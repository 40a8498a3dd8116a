// forces.cu — LJsCut and two-pass EAM force stages on the Verlet list.
//
// FP64 form: the reference's per-atom arithmetic (LJs-cut.cxx:22-131,
// EAM.cxx:141-601) including the Periodic boundary's ghost pass
// (boundary/periodic.cxx:36-102): listed pairs contribute with the raw
// difference r_j - r_i; for atoms flagged by Periodic::prepare_one, listed
// pairs at raw distance >= max(rns) contribute again through the shortest
// periodic image, as ghost copies at r_i + shortest(d).
//
// Mixed form: pair vectors come from FP32 offsets to the cell centres plus
// the image's cell offset stored in the list entry (minimum image, which is
// what the ghost pass produces whenever every periodic box edge is at least
// 2*rns), pair math and splines in FP32 (cubic coefficients per table
// interval), and per-atom sums with Kahan compensation.
//
// One thread per atom over the ELL list (entry k of atom i at nbr[k*np+i]),
// so the per-atom sums need no atomics and are deterministic.
#include <cuda_runtime.h>

#include "mdg_host.h"

namespace mdg {

struct FArgs {
    int n, np;
    const double *rx, *ry, *rz, *rns;
    const uint32_t *nbr, *ncnt;
    const uint16_t *kind, *tag;
    const uint8_t* bc;
    double L[3];
    int periodic[3];
    float csf[3];
    // outputs / intermediate
    double *fx, *fy, *fz;
    float *gx, *gy, *gz;  // mixed forces
    double* nc;
    double* Fp64;
    float* Fp32;
    const float4* pos32;
    float4* pos32b;
    double *Ep, *Em;
    double* V[9];
    DevStatus* st;
};

// ---------------------------------------------------------------------------
// FP64 spline pieces (EAM.cxx, same operation order)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double eam_rho64(const PotParams& P, double R1) {
    double RN = R1 * P.dr1;
    int N1 = (int)trunc(RN);
    if (N1 < P.Nr1) {
        double VR = N1;
        double DV = RN - VR;
        RN = R1 - VR * P.dr;
        VR = (P.Rho[N1 + 1] - P.Rho[N1]) * P.dr1;
        double aa = (P.dRho[N1 + 1] - VR) - (VR - P.dRho[N1]);
        double bb = aa - (VR - P.dRho[N1]);
        return P.Rho[N1] + RN * (P.dRho[N1] + DV * (DV * aa - bb));
    }
    return 0.0;
}

__device__ __forceinline__ void eam_embed64(const PotParams& P, double nr, double* EF, double* dF,
                                            DevStatus* st) {
    double RN = nr * P.drh1;
    int N1 = (int)trunc(RN);
    double dF0 = 0.0;  // the reference's output array is zero-initialised
    if (RN >= 0.0 && N1 < P.Nrh1) {
        if (N1 == P.Nrh1 - 1) atomicOr(&st->flags, FLAG_TABLE);
        double VR = N1;
        double DV = RN - VR;
        RN = nr - VR * P.drh;
        VR = (P.Femb[N1 + 1] - P.Femb[N1]) * P.drh1;
        double aa = (P.dFemb[N1 + 1] - VR) - (VR - P.dFemb[N1]);
        double bb = aa - (VR - P.dFemb[N1]);
        aa = aa * DV;
        *EF = P.Femb[N1] + RN * (P.dFemb[N1] + DV * (aa - bb));
        *dF = P.dFemb[N1] + 2.0 * DV * (1.5 * aa - bb);
    } else {
        atomicOr(&st->flags, FLAG_TABLE);
        if (N1 >= P.Nrh1) {
            *EF = P.Femb[P.Nrh1] + P.dFemb[P.Nrh1] * (dF0 - P.Nrh1 * P.drh);
            *dF = P.dFemb[P.Nrh1];
        } else {
            *EF = P.Femb[0] - P.dFemb[0] * dF0;
            *dF = P.dFemb[0];
        }
    }
}

// Force(r)/r of one pair and the pair energy term V(r) (EAM.cxx:417-463).
__device__ __forceinline__ double eam_ff64(const PotParams& P, double R2, double AdF, double* Vr) {
    double R1 = sqrt(R2);
    double RN = R1 * P.dr1;
    int N1 = (int)trunc(RN);
    double FF, VR, DV;
    if (N1 < P.Nr1) {
        VR = N1;
        DV = RN - VR;
        RN = R1 - VR * P.dr;
        VR = (P.Rho[N1 + 1] - P.Rho[N1]) * P.dr1;
        double aa = (P.dRho[N1 + 1] - VR) - (VR - P.dRho[N1]);
        double bb = aa - (VR - P.dRho[N1]);
        FF = P.dRho[N1] + 2.0 * DV * (1.5 * DV * aa - bb);
        VR = (P.Vpar[N1 + 1] - P.Vpar[N1]) * P.dr1;
        aa = (P.dVpar[N1 + 1] - VR) - (VR - P.dVpar[N1]);
        bb = aa - (VR - P.dVpar[N1]);
        aa = aa * DV;
        VR = P.Vpar[N1] + RN * (P.dVpar[N1] + DV * (aa - bb));
        DV = P.dVpar[N1] + 2.0 * DV * (1.5 * aa - bb);
    } else {
        FF = 0.0;
        VR = 0.0;
        DV = 0.0;
    }
    if (Vr) *Vr = 0.5 * VR / R1;
    return (AdF * FF + (DV * R1 - VR) / R2) / R1;
}

__device__ __forceinline__ double lj_pref64(const PotParams& P, double r2) {
    double r2inv = 1.0 / r2;
    double r6inv = r2inv * r2inv * r2inv;
    return -0.5 * P.factor * (P.lj1 * r6inv - P.lj2) * r6inv * r2inv;
}

// Visits the listed pairs of atom i the way Pair::* + Periodic::*_one do:
// main pass with raw differences, then the ghost pass for bc atoms.
// fn(kj, j, dx, dy, dz, r2, ghost)
template <bool MULTI, typename Fn>
__device__ __forceinline__ void visit64(const FArgs& A, int i, Fn&& fn) {
    double xi = A.rx[i], yi = A.ry[i], zi = A.rz[i];
    int cnt = A.ncnt[i];
    // main pass (the self entry contributes nothing: r2 < 1e-15)
    for (int k = 0; k < cnt; ++k) {
        uint32_t j = A.nbr[nidx(k, i, A.np)] & kJMask;
        int kj = MULTI ? (A.kind[j] & 3) : 0;
        double dx = A.rx[j] - xi, dy = A.ry[j] - yi, dz = A.rz[j] - zi;
        double r2 = dx * dx + dy * dy + dz * dz;
        fn(kj, (int)j, dx, dy, dz, r2, false);
    }
    if (!A.bc[i]) return;
    double rni = A.rns[i];
    for (int k = 0; k < cnt; ++k) {
        uint32_t j = A.nbr[nidx(k, i, A.np)] & kJMask;
        int kj = MULTI ? (A.kind[j] & 3) : 0;
        double dx = A.rx[j] - xi, dy = A.ry[j] - yi, dz = A.rz[j] - zi;
        double rnj = A.rns[j];
        double r2rns = rnj < rni ? rni : rnj;
        r2rns *= r2rns;
        if (dx * dx + dy * dy + dz * dz < r2rns) continue;
        dx = shortest1(dx, A.L[0], A.periodic[0]);
        dy = shortest1(dy, A.L[1], A.periodic[1]);
        dz = shortest1(dz, A.L[2], A.periodic[2]);
        if (dx * dx + dy * dy + dz * dz > r2rns) continue;
        // ghost copy at r_i + d, seen from r_i
        double gx = (xi + dx) - xi, gy = (yi + dy) - yi, gz = (zi + dz) - zi;
        double r2 = gx * gx + gy * gy + gz * gz;
        fn(kj, (int)j, gx, gy, gz, r2, true);
    }
}

// ---- LJsCut / EAM forces, FP64 ------------------------------------------------
template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_forces64(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    int ki = MULTI ? (A.kind[i] & 3) : 0;
    double fm[3] = {0, 0, 0}, fg[3] = {0, 0, 0};
    const int nk = ps->nkinds;
    visit64<MULTI>(A, i, [&](int kj, int j, double dx, double dy, double dz, double r2, bool ghost) {
        const PotParams& P = ps->p[ki][kj];
        if (r2 > P.R2cut || r2 < 1e-15) return;
        double pref;
        if (P.type == 1) {
            pref = lj_pref64(P, r2);
        } else if (P.type == 2) {
            double AdF = A.Fp64[(size_t)ki * A.np + j] + A.Fp64[(size_t)kj * A.np + i];
            pref = eam_ff64(P, r2, AdF, nullptr);
        } else {
            return;
        }
        double* f = ghost ? fg : fm;
        f[0] += dx * pref;
        f[1] += dy * pref;
        f[2] += dz * pref;
    });
    (void)nk;
    double fx = fm[0] + fg[0], fy = fm[1] + fg[1], fz = fm[2] + fg[2];
    if (!isfinite(fx) || !isfinite(fy) || !isfinite(fz)) atomicOr(&A.st->flags, FLAG_NONFINITE);
    A.fx[i] = fx;
    A.fy[i] = fy;
    A.fz[i] = fz;
}

// ---- EAM density + embedding derivative, FP64 ------------------------------
template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_density64(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    if (A.tag[i] == 0) {
        // untouched by the reference's charge stage; F' still defined
        double nci = A.nc[i];
        int ki = MULTI ? (A.kind[i] & 3) : 0;
        for (int b = 0; b < ps->nkinds; ++b) {
            const PotParams& P = ps->p[ki][b];
            double EF = 0, dF = 0;
            if (P.type == 2) eam_embed64(P, nci, &EF, &dF, A.st);
            A.Fp64[(size_t)b * A.np + i] = dF;
        }
        return;
    }
    int ki = MULTI ? (A.kind[i] & 3) : 0;
    double sm = 0.0, sg = 0.0;
    visit64<MULTI>(A, i, [&](int kj, int j, double, double, double, double r2, bool ghost) {
        const PotParams& P = ps->p[ki][kj];
        if (P.type != 2 || r2 > P.R2cut || r2 < 1e-15) return;
        double v = eam_rho64(P, sqrt(r2));
        if (ghost) sg = sg + v;
        else sm = sm + v;
    });
    double nci = sm + sg;
    A.nc[i] = nci;
    for (int b = 0; b < ps->nkinds; ++b) {
        const PotParams& P = ps->p[ki][b];
        double EF = 0, dF = 0;
        if (P.type == 2) eam_embed64(P, nci, &EF, &dF, A.st);
        A.Fp64[(size_t)b * A.np + i] = dF;
    }
}

// ---- energies and virials, FP64 (LJs-cut.cxx:70-131, EAM.cxx:306-415) ------
template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_virials64(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    int ki = MULTI ? (A.kind[i] & 3) : 0;
    double Ep = 0.0;
    double M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int last_kind = -1;
    visit64<MULTI>(A, i, [&](int kj, int j, double dx, double dy, double dz, double r2, bool ghost) {
        const PotParams& P = ps->p[ki][kj];
        if (P.type == 2) last_kind = kj > last_kind || ghost ? kj : last_kind;
        if (r2 > P.R2cut || r2 < 1e-15) return;
        double d[3] = {dx, dy, dz};
        if (P.type == 1) {
            double r2inv = 1.0 / r2;
            double r6inv = r2inv * r2inv * r2inv;
            double pref = -0.5 * P.factor * (P.lj1 * r6inv - P.lj2) * r6inv * r2inv;
            double tmp = P.s6 * r6inv;
            Ep += 0.5 * 4 * P.a * tmp * (tmp - 1);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) M[r + 3 * c] += 0.5 * (pref * d[r]) * d[c];
        } else if (P.type == 2) {
            double AdF = A.Fp64[(size_t)ki * A.np + j] + A.Fp64[(size_t)kj * A.np + i];
            double Vr;
            double FF = eam_ff64(P, r2, AdF, &Vr);
            double h = 0.5 * FF;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) M[r + 3 * c] += h * d[r] * d[c];
            Ep += Vr;
        }
    });
    A.Ep[i] = Ep;
    for (int k = 0; k < 9; ++k) A.V[k][i] = M[k];
    if (ps->any_eam) {
        int kb = MULTI ? (last_kind >= 0 ? last_kind : ki) : 0;
        const PotParams& P = ps->p[ki][kb];
        double EF = 0.0, dF = 0.0;
        if (P.type == 2) {
            eam_embed64(P, A.nc[i], &EF, &dF, A.st);
            A.Em[i] = EF;
        }
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

// Pair vector r_j - r_i of a list entry, from cell-centred offsets.
__device__ __forceinline__ void pair_vec32(uint32_t e, const float4& pi, const float4& pj,
                                           const float csf[3], float& dx, float& dy, float& dz) {
    dx = (pj.x - pi.x) + image_shift(e, 0, csf[0]);
    dy = (pj.y - pi.y) + image_shift(e, 1, csf[1]);
    dz = (pj.z - pi.z) + image_shift(e, 2, csf[2]);
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

// The pair loops below read four list entries with one 16-byte load, then
// the four neighbour records, so the loads of a group overlap; the four
// contributions are summed in FP32 and the group sum enters a Kahan sum.

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_lj_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    const float4 pi = A.pos32[i];
    const int ng = A.ncnt[i] >> 2;
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const bool per = ps->periodic;
    const float csf[3] = {A.csf[0], A.csf[1], A.csf[2]};
    const PotParams& P0 = ps->p[ki][0];
    float r2c = P0.r2cut_f, l1 = P0.lj1_f, l2 = P0.lj2_f, mh = P0.mhf_f;
    double R2c = P0.R2cut;
    Kahan3 acc;
    const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
    for (int g = 0; g < ng; ++g) {
        const uint4 e4 = __ldg(row + (size_t)g * A.np);
        const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
        float4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32 + (e[q] & kJMask));
        float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (MULTI) {
                const PotParams& P = ps->p[ki][A.kind[e[q] & kJMask] & 3];
                r2c = P.r2cut_f; l1 = P.lj1_f; l2 = P.lj2_f; mh = P.mhf_f; R2c = P.R2cut;
            }
            float dx, dy, dz;
            pair_vec32(e[q], pi, pj[q], csf, dx, dy, dz);
            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool in = pair_in(A, i, e[q], r2, r2c, R2c, per);
            float r2inv = __frcp_rn(fmaxf(r2, 1e-12f));
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
    A.gx[i] = acc.s[0];
    A.gy[i] = acc.s[1];
    A.gz[i] = acc.s[2];
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

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_density_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const float4 pi = A.pos32[i];
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const float csf[3] = {A.csf[0], A.csf[1], A.csf[2]};
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
        for (int g = 0; g < ng; ++g) {
            const uint4 e4 = __ldg(row + (size_t)g * A.np);
            const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
            float4 pj[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32 + (e[q] & kJMask));
            float part = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                bool eam = true;
                if (MULTI) {
                    P = &ps->p[ki][A.kind[e[q] & kJMask] & 3];
                    r2c = P->r2cut_f; idr = P->inv_dr_f; Nr1 = P->Nr1; tab = P->rho_c; R2c = P->R2cut;
                    eam = P->type == 2;
                }
                float dx, dy, dz;
                pair_vec32(e[q], pi, pj[q], csf, dx, dy, dz);
                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                bool in = eam && pair_in(A, i, e[q], r2, r2c, R2c, per);
                float t = sqrtf(r2) * idr;
                int nn = (int)t;
                in = in && nn < Nr1;
                nn = in ? nn : 0;
                float u = t - (float)nn;
                float v = in ? cubic(__ldg(tab + nn), u) : 0.f;
                part += v;
            }
            ksum_add(s, c, part);
        }
    }
    float rho = s;
    float Fp0 = 0.f;
    for (int b = 0; b < ps->nkinds; ++b) {
        const PotParams& P = ps->p[ki][b];
        float F = 0.f, dF = 0.f;
        if (P.type == 2) embed32(P, rho, &F, &dF, A.st);
        if (b == 0) Fp0 = dF;
        if (MULTI) A.Fp32[(size_t)b * A.np + i] = dF;
    }
    A.pos32b[i] = make_float4(pi.x, pi.y, pi.z, Fp0);
}

template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_eam_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    const float4 pi = A.pos32b[i];
    const int ng = A.ncnt[i] >> 2;
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    const float csf[3] = {A.csf[0], A.csf[1], A.csf[2]};
    const bool per = ps->periodic;
    const PotParams* P = &ps->p[ki][0];
    float r2c = P->r2cut_f, idr = P->inv_dr_f;
    double R2c = P->R2cut;
    int Nr1 = P->Nr1;
    const float4* rt = P->rho_c;
    const float4* vt = P->v_c;
    Kahan3 acc;
    const uint4* row = reinterpret_cast<const uint4*>(A.nbr) + i;
    for (int g = 0; g < ng; ++g) {
        const uint4 e4 = __ldg(row + (size_t)g * A.np);
        const uint32_t e[4] = {e4.x, e4.y, e4.z, e4.w};
        float4 pj[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) pj[q] = __ldg(A.pos32b + (e[q] & kJMask));
        float fx = 0.f, fy = 0.f, fz = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float Fpi = pi.w, Fpj = pj[q].w;
            bool eam = true;
            if (MULTI) {
                uint32_t j = e[q] & kJMask;
                int kj = A.kind[j] & 3;
                P = &ps->p[ki][kj];
                eam = P->type == 2;
                r2c = P->r2cut_f; idr = P->inv_dr_f; Nr1 = P->Nr1; rt = P->rho_c; vt = P->v_c; R2c = P->R2cut;
                Fpj = A.Fp32[(size_t)ki * A.np + j];
                Fpi = A.Fp32[(size_t)kj * A.np + i];
            }
            float dx, dy, dz;
            pair_vec32(e[q], pi, pj[q], csf, dx, dy, dz);
            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            bool in = eam && pair_in(A, i, e[q], r2, r2c, R2c, per);
            float r = sqrtf(r2);
            float t = r * idr;
            int nn = (int)t;
            in = in && nn < Nr1;
            nn = in ? nn : 0;
            float u = t - (float)nn;
            float4 cr = __ldg(rt + nn);
            float4 cv = __ldg(vt + nn);
            float drho = dcubic(cr, u) * idr;
            float V = cubic(cv, u);
            float dV = dcubic(cv, u) * idr;
            float rinv = __frcp_rn(fmaxf(r, 1e-6f));
            float FF = fmaf(Fpi + Fpj, drho, (dV * r - V) * (rinv * rinv)) * rinv;
            FF = in ? FF : 0.f;
            fx = fmaf(FF, dx, fx);
            fy = fmaf(FF, dy, fy);
            fz = fmaf(FF, dz, fz);
        }
        acc.add(0, fx);
        acc.add(1, fy);
        acc.add(2, fz);
    }
    A.gx[i] = acc.s[0];
    A.gy[i] = acc.s[1];
    A.gz[i] = acc.s[2];
}


// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

static FArgs make_args(mdg_system* sys) {
    FArgs A;
    memset(&A, 0, sizeof(A));
    int c = sys->cur;
    A.n = (int)sys->n;
    A.np = (int)sys->np;
    A.rx = sys->f64[RX][c];
    A.ry = sys->f64[RY][c];
    A.rz = sys->f64[RZ][c];
    A.rns = sys->f64[RNS][c];
    A.nbr = sys->nbr;
    A.ncnt = sys->ncnt;
    A.kind = sys->u16[KIND][c];
    A.tag = sys->u16[TAG][c];
    A.bc = sys->bc;
    for (int a = 0; a < 3; ++a) {
        A.L[a] = sys->dom.bmax[a] - sys->dom.bmin[a];
        A.periodic[a] = sys->dom.periodic[a] ? 1 : 0;
        A.csf[a] = sys->grid.csf[a];
    }
    A.fx = sys->f64[FX][c];
    A.fy = sys->f64[FY][c];
    A.fz = sys->f64[FZ][c];
    A.gx = sys->f32[0][c];
    A.gy = sys->f32[1][c];
    A.gz = sys->f32[2][c];
    A.nc = sys->f64[NC][c];
    A.Fp64 = sys->Fp64;
    A.Fp32 = sys->Fp32;
    A.pos32 = sys->pos32;
    A.pos32b = reinterpret_cast<float4*>(sys->pos32 + sys->np);
    A.Ep = sys->f64[EP][c];
    A.Em = sys->f64[EM][c];
    for (int k = 0; k < 9; ++k) A.V[k] = sys->f64[V0 + k][c];
    A.st = sys->dstat;
    return A;
}

// stage: 0 = charge (density), 1 = forces
int launch_stage(mdg_system* sys, const PotSet* dps, const PotSet& ps, int precision, int stage) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    FArgs A = make_args(sys);
    int nb = nblk(sys->n);
    if (sys->n == 0) return MDG_OK;
    bool multi = ps.multi != 0;
    if (precision == MDG_PREC_FP64) {
        if (stage == 0) {
            if (multi) k_density64<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_density64<false><<<nb, kBlock, 0, st>>>(A, dps);
        } else {
            if (multi) k_forces64<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_forces64<false><<<nb, kBlock, 0, st>>>(A, dps);
        }
    } else {
        if (stage == 0) {
            if (multi) k_density_mixed<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_density_mixed<false><<<nb, kBlock, 0, st>>>(A, dps);
        } else if (ps.any_eam) {
            if (multi) k_eam_mixed<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_eam_mixed<false><<<nb, kBlock, 0, st>>>(A, dps);
        } else {
            if (multi) k_lj_mixed<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_lj_mixed<false><<<nb, kBlock, 0, st>>>(A, dps);
        }
    }
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

int launch_virials(mdg_system* sys, const PotSet* dps, const PotSet& ps) {
    mdg_ctx* ctx = sys->ctx;
    if (sys->n == 0) return MDG_OK;
    FArgs A = make_args(sys);
    int nb = nblk(sys->n);
    if (ps.multi) k_virials64<true><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
    else k_virials64<false><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

}  // namespace mdg
