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

#include <algorithm>
#include <cstring>

#include "mdg_host.h"
#include "forces_dev.cuh"
#include "integrate_dev.cuh"

namespace mdg {


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

// Force(r)/r of a tabulated Pair and its energy term V(r)/(2r)
// (pair.cxx:316-346, 228-314).
__device__ __forceinline__ double tab_ff64(const PotParams& P, double R2, double* Vr) {
    double R1 = sqrt(R2);
    double RN = R1 * P.dr1;
    int N1 = (int)trunc(RN);
    double VR = 0.0, DV = 0.0;
    if (N1 < P.Nr1) {
        VR = N1;
        DV = RN - VR;
        RN = R1 - VR * P.dr;
        VR = (P.Vpar[N1 + 1] - P.Vpar[N1]) * P.dr1;
        double aa = (P.dVpar[N1 + 1] - VR) - (VR - P.dVpar[N1]);
        double bb = aa - (VR - P.dVpar[N1]);
        aa = aa * DV;
        VR = P.Vpar[N1] + RN * (P.dVpar[N1] + DV * (aa - bb));
        DV = P.dVpar[N1] + 2.0 * DV * (1.5 * aa - bb);
    }
    if (Vr) *Vr = 0.5 * VR / R1;
    return ((DV * R1 - VR) / R2) / R1;
}

// LJs force / r (LJs.cxx:153-166) and energy term (LJs.cxx:90-101).
__device__ __forceinline__ double ljs_ff64(const PotParams& P, double r2, double* E) {
    const double X2min = 1.2599210498948732;
    double XX = P.ljs_rVr1 * r2 - X2min;
    double FV = P.ljs_rVr2 / r2;
    double Ur = FV * FV * FV;
    if (E) *E = P.ljs_aVr * (Ur * (Ur - 1.0) - (P.ljs_aLJ3 + P.ljs_bLJ2 * XX) * XX * XX);
    return P.ljs_aVr2 * (Ur * (Ur - 0.5) * FV + (P.ljs_aLJ + P.ljs_bLJ * XX) * XX);
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

// ---- F'(nc) of the current densities, FP64 -----------------------------------
// The reference's force pass evaluates the embedding derivative from each
// atom's nc as it is (EAM.cxx:465-497); the FP64 force kernel reads it from
// Fp64, which the density pass writes. When nc changed since (prepare clears
// it, an upload replaces it, a rebuild permutes the atoms), this pass brings
// Fp64 back in line before a force pass.
template <bool MULTI>
__global__ void __launch_bounds__(kBlock) k_embed64(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const double nci = A.nc[i];
    const int ki = MULTI ? (A.kind[i] & 3) : 0;
    for (int b = 0; b < ps->nkinds; ++b) {
        const PotParams& P = ps->p[ki][b];
        double EF = 0, dF = 0;
        if (P.type == 2) eam_embed64(P, nci, &EF, &dF, A.st);
        A.Fp64[(size_t)b * A.np + i] = dF;
    }
}

// ---- LJsCut / EAM forces, FP64 ------------------------------------------------
// HALF (half lists, verlet-list.cxx:345): the pair-type potentials push the
// pair force onto the neighbour as well (LJs-cut.cxx:57-62, pair.cxx:387-420,
// LJs.cxx:196-222); EAM uses the atom's half alone, as EAM::force does; the
// ghost pass acts on the atom alone (its ghost list is a full one,
// periodic.cxx:77-88). Both sides accumulate with atomics onto the outputs
// prepare cleared, as the reference's += does.
template <bool MULTI, bool HALF>
__global__ void __launch_bounds__(kBlock) k_forces64(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    int ki = MULTI ? (A.kind[i] & 3) : 0;
    double fm[3] = {0, 0, 0}, fg[3] = {0, 0, 0};
    visit64<MULTI>(A, i, [&](int kj, int j, double dx, double dy, double dz, double r2, bool ghost) {
        const PotParams& P = ps->p[ki][kj];
        if (r2 > P.R2cut || r2 < 1e-15) return;
        double pref;
        if (P.type == 1) {
            pref = lj_pref64(P, r2);
        } else if (P.type == 2) {
            double AdF = A.Fp64[(size_t)ki * A.np + j] + A.Fp64[(size_t)kj * A.np + i];
            pref = eam_ff64(P, r2, AdF, nullptr);
        } else if (P.type == POT_TAB) {
            pref = tab_ff64(P, r2, nullptr);
        } else if (P.type == POT_LJS) {
            pref = ljs_ff64(P, r2, nullptr);
        } else {
            return;
        }
        double* f = ghost ? fg : fm;
        f[0] += dx * pref;
        f[1] += dy * pref;
        f[2] += dz * pref;
        if (HALF && !ghost && P.type != 2) {
            atomicAdd(&A.fx[j], -(dx * pref));
            atomicAdd(&A.fy[j], -(dy * pref));
            atomicAdd(&A.fz[j], -(dz * pref));
        }
    });
    double fx = fm[0] + fg[0], fy = fm[1] + fg[1], fz = fm[2] + fg[2];
    if (!isfinite(fx) || !isfinite(fy) || !isfinite(fz)) atomicOr(&A.st->flags, FLAG_NONFINITE);
    if (HALF) {
        atomicAdd(&A.fx[i], fx);
        atomicAdd(&A.fy[i], fy);
        atomicAdd(&A.fz[i], fz);
    } else {
        A.fx[i] = fx;
        A.fy[i] = fy;
        A.fz[i] = fz;
    }
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

// ---- energies and virials, FP64 (LJs-cut.cxx:70-131, EAM.cxx:306-415,
// pair.cxx:228-314, LJs.cxx:103-151); HALF as for the forces above.
template <bool MULTI, bool HALF>
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
        double E = 0.0, Mp[9];
        if (P.type == 1) {
            double r2inv = 1.0 / r2;
            double r6inv = r2inv * r2inv * r2inv;
            double pref = -0.5 * P.factor * (P.lj1 * r6inv - P.lj2) * r6inv * r2inv;
            double tmp = P.s6 * r6inv;
            E = 0.5 * 4 * P.a * tmp * (tmp - 1);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Mp[r + 3 * c] = 0.5 * (pref * d[r]) * d[c];
        } else if (P.type == 2) {
            double AdF = A.Fp64[(size_t)ki * A.np + j] + A.Fp64[(size_t)kj * A.np + i];
            double FF = eam_ff64(P, r2, AdF, &E);
            double h = 0.5 * FF;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Mp[r + 3 * c] = h * d[r] * d[c];
        } else if (P.type == POT_TAB) {
            double h = 0.5 * tab_ff64(P, r2, &E);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Mp[r + 3 * c] = h * d[r] * d[c];
        } else if (P.type == POT_LJS) {
            double FF = ljs_ff64(P, r2, &E);
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) Mp[r + 3 * c] = 0.5 * (FF * d[r]) * d[c];
        } else {
            return;
        }
        Ep += E;
        for (int k = 0; k < 9; ++k) M[k] += Mp[k];
        if (HALF && !ghost && P.type != 2) {
            atomicAdd(&A.Ep[j], E);
            for (int k = 0; k < 9; ++k) atomicAdd(&A.V[k][j], Mp[k]);
        }
    });
    if (HALF) {
        atomicAdd(&A.Ep[i], Ep);
        for (int k = 0; k < 9; ++k) atomicAdd(&A.V[k][i], M[k]);
    } else {
        A.Ep[i] = Ep;
        for (int k = 0; k < 9; ++k) A.V[k][i] = M[k];
    }
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
// mixed precision (bodies in forces_dev.cuh)
// ---------------------------------------------------------------------------
// Blocks of 256 threads per SM the register budget must allow, measured on
// EAM Cu 1M atoms: the force pass is fastest at 4 (64 registers; 0.227 ms
// against 0.237 ms at 3), the density pass at 4 (0.165 ms against 0.177 ms
// at 5, where it spills).
constexpr int kForceMinBlocks = 4;
constexpr int kDensityMinBlocks = 4;
// The Multi force body (per-pair kind, parameters and F' columns) spills at
// 64 registers; three blocks per SM (up to 85 registers) measured fastest on
// NiAl B2 1M atoms: 7.2e8 atom-steps/s against 6.4e8 at four blocks and
// 6.2e8 at two. The Multi density body fits 64 registers without spills and
// runs best at four blocks like the single one (7.39e8 against 7.20e8).
constexpr int kMultiMinBlocks = 3;
// MB = blocks of 256 threads per SM the register budget allows: a system's
// launch shape (mdg_system_set_shape, chosen by the project's autotuner),
// default as above.
template <bool MULTI, bool KICK, int MB>
__global__ void __launch_bounds__(kBlock, MB) k_lj_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) lj_mixed_one<MULTI, KICK>(A, ps, i);
}

template <bool MULTI, int MB>
__global__ void __launch_bounds__(kBlock, MB) k_density_rec(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) density_mixed_one<MULTI, true>(A, ps, i);
}

template <bool MULTI, int MB>
__global__ void __launch_bounds__(kBlock, MB) k_density_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) density_mixed_one<MULTI>(A, ps, i);
}

template <bool MULTI, bool KICK, int MB>
__global__ void __launch_bounds__(kBlock, MB) k_eam_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) eam_mixed_one<MULTI, KICK>(A, ps, i);
}

// The blocks-per-SM budget of a pass: the system's shape if set, else the
// measured default for its form.
static int force_blocks(const mdg_system* sys, bool multi) {
    return sys->shape[MDG_SHAPE_FORCE_BLOCKS_PER_SM] ? sys->shape[MDG_SHAPE_FORCE_BLOCKS_PER_SM]
                                                     : (multi ? kMultiMinBlocks : kForceMinBlocks);
}
static int density_blocks(const mdg_system* sys, bool multi) {
    (void)multi;  // the Multi body fits the same budget
    return sys->shape[MDG_SHAPE_DENSITY_BLOCKS_PER_SM] ? sys->shape[MDG_SHAPE_DENSITY_BLOCKS_PER_SM]
                                                       : kDensityMinBlocks;
}

template <bool MULTI, bool KICK>
static void launch_eam_lj(bool eam, int mb, const FArgs& A, const PotSet* dps, int nb, cudaStream_t st) {
    if (eam) {
        if (mb == 3) k_eam_mixed<MULTI, KICK, 3><<<nb, kBlock, 0, st>>>(A, dps);
        else k_eam_mixed<MULTI, KICK, 4><<<nb, kBlock, 0, st>>>(A, dps);
    } else {
        if (mb == 3) k_lj_mixed<MULTI, KICK, 3><<<nb, kBlock, 0, st>>>(A, dps);
        else k_lj_mixed<MULTI, KICK, 4><<<nb, kBlock, 0, st>>>(A, dps);
    }
}

template <bool MULTI>
static void launch_density(int mb, const FArgs& A, const PotSet* dps, int nb, cudaStream_t st) {
    if (mb == 3) k_density_mixed<MULTI, 3><<<nb, kBlock, 0, st>>>(A, dps);
    else if (mb == 5) k_density_mixed<MULTI, 5><<<nb, kBlock, 0, st>>>(A, dps);
    else k_density_mixed<MULTI, 4><<<nb, kBlock, 0, st>>>(A, dps);
}


template <bool MULTI, int FORM, bool KICK>
__global__ void __launch_bounds__(kBlock, kForceMinBlocks) k_pair_mixed(FArgs A, const PotSet* __restrict__ ps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) pair_mixed_one<MULTI, FORM, KICK>(A, ps, i);
}

// ---- Langevin thermostat (langevin.cxx:29-42) ----------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): ten rounds of two
// 32x32->64 multiplications, key bumped by the Weyl constants.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

struct ThermoArgs {
    int n;
    const double *rx, *vx, *vy, *vz, *m;
    const uint32_t* orig;
    double *fx, *fy, *fz;  // FP64 form
    float *gx, *gy, *gz;   // mixed form
    const DevStatus* st;
};

// f += heat * (sqrt(m) * sigma * z - (v - U) * beta * m) for every term whose
// x range holds the atom; z = three Box-Muller normals of one Philox block
// with counter {caller index, call number, term, 0}.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_langevin(ThermoArgs A, const ThermoDev* __restrict__ th) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const int nt = th->n;
    if (nt == 0) return;
    const uint32_t call = A.st->therm_calls;
    const double x = A.rx[i], m = A.m[i];
    const double v[3] = {A.vx[i], A.vy[i], A.vz[i]};
    const double sqrt_mass = sqrt(m);
    double f[3] = {0.0, 0.0, 0.0};
    if (!MIXED) {
        f[0] = A.fx[i];
        f[1] = A.fy[i];
        f[2] = A.fz[i];
    }
    const uint32_t atom = A.orig[i];
    for (int q = 0; q < nt && q < kMaxThermo; ++q) {
        const LangevinTerm& L = th->t[q];
        if (x < L.xmin || x > L.xmax) continue;
        const uint4 b = philox4x32_10(make_uint4(atom, call, (uint32_t)q, 0u),
                                      make_uint2((uint32_t)L.seed, (uint32_t)(L.seed >> 32)));
        const double k32 = 2.3283064365386962890625e-10;  // 2^-32
        const double two_pi = 6.283185307179586476925;
        const double ra = sqrt(-2.0 * log(((double)b.x + 0.5) * k32));
        const double rb = sqrt(-2.0 * log(((double)b.z + 0.5) * k32));
        const double a1 = two_pi * (((double)b.y + 0.5) * k32);
        const double a3 = two_pi * (((double)b.w + 0.5) * k32);
        const double z[3] = {ra * cos(a1), ra * sin(a1), rb * cos(a3)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double tf = __dmul_rn(__dadd_rn(__dmul_rn(z[k], L.sigma), 0.0), sqrt_mass);
            tf = __dsub_rn(tf, __dmul_rn(__dmul_rn(__dsub_rn(v[k], L.U[k]), L.beta), m));
            tf = __dmul_rn(tf, L.heat[k]);
            f[k] = __dadd_rn(f[k], tf);
        }
    }
    if (MIXED) {
        A.gx[i] += (float)f[0];
        A.gy[i] += (float)f[1];
        A.gz[i] += (float)f[2];
    } else {
        A.fx[i] = f[0];
        A.fy[i] = f[1];
        A.fz[i] = f[2];
    }
}

__global__ void k_thermo_tick(DevStatus* st) {
    if (threadIdx.x == 0) st->therm_calls += 1u;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

FArgs force_args(mdg_system* sys) {
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
        A.uf[a] = (float)(sys->grid.cs[a] / kOffUnits);
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
    A.pos32b = sys->pos32 + sys->np;
    A.cutbits = nullptr;  // set by the passes of a step loop whose force pass moves atoms
    A.Ep = sys->f64[EP][c];
    A.Em = sys->f64[EM][c];
    for (int k = 0; k < 9; ++k) A.V[k] = sys->f64[V0 + k][c];
    A.st = sys->dstat;
    A.m = sys->f64[MASS][c];
    A.vx = sys->f64[VX][c];
    A.vy = sys->f64[VY][c];
    A.vz = sys->f64[VZ][c];
    A.kick_hdt = 0.0f;
    return A;
}

// Thermostat pass after the force stage (pair.cxx:81), then the call
// counter's increment.
static int launch_thermostat(mdg_system* sys, const ThermoDev* th, int precision) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    int c = sys->cur;
    ThermoArgs T;
    T.n = (int)sys->n;
    T.rx = sys->f64[RX][c];
    T.vx = sys->f64[VX][c];
    T.vy = sys->f64[VY][c];
    T.vz = sys->f64[VZ][c];
    T.m = sys->f64[MASS][c];
    T.orig = sys->u32[ORIG][c];
    T.fx = sys->f64[FX][c];
    T.fy = sys->f64[FY][c];
    T.fz = sys->f64[FZ][c];
    T.gx = sys->f32[0][c];
    T.gy = sys->f32[1][c];
    T.gz = sys->f32[2][c];
    T.st = sys->dstat;
    int nb = nblk(sys->n);
    if (precision == MDG_PREC_FP64) k_langevin<false><<<nb, kBlock, 0, st>>>(T, th);
    else k_langevin<true><<<nb, kBlock, 0, st>>>(T, th);
    MDG_LAUNCHED(ctx);
    k_thermo_tick<<<1, 32, 0, st>>>(sys->dstat);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

template <bool KICK>
static void launch_forces_mixed(const mdg_system* sys, const FArgs& A, const PotSet* dps, const PotSet& ps, int nb,
                                cudaStream_t st) {
    const bool multi = ps.multi != 0;
    const int mb = force_blocks(sys, multi);
    if (ps.any_eam) {
        if (multi) launch_eam_lj<true, KICK>(true, mb, A, dps, nb, st);
        else launch_eam_lj<false, KICK>(true, mb, A, dps, nb, st);
    } else if (ps.any_tab || ps.any_ljs) {
        const int kinds = ps.any_lj + ps.any_tab + ps.any_ljs;
        if (!multi && ps.any_tab) k_pair_mixed<false, 3, KICK><<<nb, kBlock, 0, st>>>(A, dps);
        else if (!multi) k_pair_mixed<false, 4, KICK><<<nb, kBlock, 0, st>>>(A, dps);
        else if (kinds > 1) k_pair_mixed<true, 0, KICK><<<nb, kBlock, 0, st>>>(A, dps);
        else if (ps.any_tab) k_pair_mixed<true, 3, KICK><<<nb, kBlock, 0, st>>>(A, dps);
        else k_pair_mixed<true, 4, KICK><<<nb, kBlock, 0, st>>>(A, dps);
    } else {
        if (multi) launch_eam_lj<true, KICK>(false, mb, A, dps, nb, st);
        else launch_eam_lj<false, KICK>(false, mb, A, dps, nb, st);
    }
}

// ---- the force pass that starts the next step -----------------------------
// The step loop's EAM force pass (mixed form, no thermostat) with the step's
// second half-kick. When the next step can start in it — steps remain after
// this one (*left > 1) and no rebuild is due at this step's positions
// (need_rebuild, from the drift that made them) — every atom then also runs
// the next step's first half-kick, drift, offsets refresh and rebuild test
// (kick_drift_mixed; atoms with tag 0 only the last two), the test's result
// into need_next; otherwise the next drift runs as its own pass after the
// rebuild. The decision is the same for every thread. Moving atoms while
// others still read them is safe here because this pass reads its
// neighbours only through the density pass's copies (pos32b, Fp32) and takes
// each pair's cut decision from the density pass (cutbits), where the
// unfused pass would settle pairs near the cutoff on the FP64 positions.
template <bool MULTI, int MB, int NT = kBlock>
__global__ void __launch_bounds__(NT, MB)
    k_force_step(FArgs A, IArgs D, const PotSet* __restrict__ ps, const unsigned long long* __restrict__ left) {
    const bool next = *left > 1ull && A.st->need_rebuild == 0u;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = false;
    if (i < A.n) {
        float fx, fy, fz;
        const bool moved = eam_mixed_force<MULTI, true>(A, ps, i, fx, fy, fz);
        if (!next) {
            if (moved) store_force<true>(A, i, fx, fy, fz);
        } else if (moved) {
            need = kick_drift_mixed(D, A.gx, A.gy, A.gz, i, fx, fy, fz);
        } else {
            const double r[3] = {D.rx[i], D.ry[i], D.rz[i]};
            need = offsets_check_mixed(D, i, r);
        }
    }
    if (next) flag_need_next(need, A.st);
}

int launch_forces_step(mdg_system* sys, const PotSet* dps, const PotSet& ps, double dt,
                       const unsigned long long* left) {
    if (sys->n == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    FArgs A = force_args(sys);
    if (!ps.any_eam || !sys->cutbits || sys->cut_words * 32 < sys->K) {
        set_error("the step-starting force pass needs an EAM solver and the density pass's cut bits");
        return MDG_ERR_STATE;
    }
    A.cutbits = sys->cutbits;
    A.kick_hdt = 0.5f * (float)dt;
    const IArgs D = integrator_args(sys, dt);
    const int nb = nblk(sys->n);
    cudaStream_t st = ctx->stream;
    const bool multi = ps.multi != 0;
    const int mb = force_blocks(sys, multi);
    // 8: eight 128-thread blocks per SM (the 4-block budget in blocks half
    // the size, so the launch's last, partly filled wave is shorter)
    const int nb128 = nblk(sys->n, 128);
    if (multi) {
        if (mb == 3) k_force_step<true, 3><<<nb, kBlock, 0, st>>>(A, D, dps, left);
        else if (mb == 8) k_force_step<true, 8, 128><<<nb128, 128, 0, st>>>(A, D, dps, left);
        else k_force_step<true, 4><<<nb, kBlock, 0, st>>>(A, D, dps, left);
    } else {
        if (mb == 3) k_force_step<false, 3><<<nb, kBlock, 0, st>>>(A, D, dps, left);
        else if (mb == 8) k_force_step<false, 8, 128><<<nb128, 128, 0, st>>>(A, D, dps, left);
        else k_force_step<false, 4><<<nb, kBlock, 0, st>>>(A, D, dps, left);
    }
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

// The density pass of a step whose force pass moves atoms (k_force_step):
// as the charge stage, recording the band pairs' FP64 decisions.
int launch_density_rec(mdg_system* sys, const PotSet* dps, const PotSet& ps) {
    if (sys->n == 0) return MDG_OK;
    FArgs A = force_args(sys);
    if (!sys->cutbits || sys->cut_words * 32 < sys->K) {
        set_error("the density pass's cut bits are not allocated");
        return MDG_ERR_STATE;
    }
    A.cutbits = sys->cutbits;
    const int nb = nblk(sys->n);
    cudaStream_t st = sys->ctx->stream;
    const bool multi = ps.multi != 0;
    const int mb = density_blocks(sys, multi);
    if (multi) {
        if (mb == 3) k_density_rec<true, 3><<<nb, kBlock, 0, st>>>(A, dps);
        else if (mb == 5) k_density_rec<true, 5><<<nb, kBlock, 0, st>>>(A, dps);
        else k_density_rec<true, 4><<<nb, kBlock, 0, st>>>(A, dps);
    } else {
        if (mb == 3) k_density_rec<false, 3><<<nb, kBlock, 0, st>>>(A, dps);
        else if (mb == 5) k_density_rec<false, 5><<<nb, kBlock, 0, st>>>(A, dps);
        else k_density_rec<false, 4><<<nb, kBlock, 0, st>>>(A, dps);
    }
    MDG_LAUNCHED(sys->ctx);
    sys->fp_ok = 0;  // nc rewritten (FP32 sums); Fp64 no longer matches it
    return MDG_OK;
}

// The density pass's cut bits of a system (mdg_system::cutbits), sized for
// its list capacity; the force pass that starts the next step reads them.
int ensure_cutbits(mdg_system* sys) {
    const int words = (sys->K + 31) / 32;
    if (sys->cutbits && sys->cut_words >= words) return MDG_OK;
    sys_free(sys, sys->cutbits, (size_t)sys->cut_words * sys->np * sizeof(uint32_t));
    sys->cutbits = nullptr;
    sys->cut_words = 0;
    int rc = sys_malloc(sys, (void**)&sys->cutbits, (size_t)std::max(words, 1) * sys->np * sizeof(uint32_t));
    if (rc) return rc;
    sys->cut_words = std::max(words, 1);
    return MDG_OK;
}

// stage: 0 = charge (density), 1 = forces (then the thermostat, if any).
// kick_dt > 0 (mixed form, force stage, no thermostat): the step's second
// half-kick is applied in the force pass.
int launch_stage(mdg_system* sys, const PotSet* dps, const PotSet& ps, int precision, int stage,
                 const ThermoDev* th, double kick_dt) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    FArgs A = force_args(sys);
    int nb = nblk(sys->n);
    if (sys->n == 0) return MDG_OK;
    bool multi = ps.multi != 0;
    if (precision == MDG_PREC_FP64) {
        if (stage == 0) {
            if (multi) k_density64<true><<<nb, kBlock, 0, st>>>(A, dps);
            else k_density64<false><<<nb, kBlock, 0, st>>>(A, dps);
            sys->fp_ok = 1;
        } else {
            if (ps.any_eam && !sys->fp_ok) {
                if (multi) k_embed64<true><<<nb, kBlock, 0, st>>>(A, dps);
                else k_embed64<false><<<nb, kBlock, 0, st>>>(A, dps);
                MDG_LAUNCHED(ctx);
                sys->fp_ok = 1;
            }
            if (sys->half) {
                if (multi) k_forces64<true, true><<<nb, kBlock, 0, st>>>(A, dps);
                else k_forces64<false, true><<<nb, kBlock, 0, st>>>(A, dps);
            } else {
                if (multi) k_forces64<true, false><<<nb, kBlock, 0, st>>>(A, dps);
                else k_forces64<false, false><<<nb, kBlock, 0, st>>>(A, dps);
            }
        }
    } else {
        if (stage == 0) {
            if (multi) launch_density<true>(density_blocks(sys, true), A, dps, nb, st);
            else launch_density<false>(density_blocks(sys, false), A, dps, nb, st);
            sys->fp_ok = 0;  // nc rewritten (FP32 sums); Fp64 no longer matches it
        } else if (kick_dt > 0.0 && !th) {
            A.kick_hdt = 0.5f * (float)kick_dt;
            launch_forces_mixed<true>(sys, A, dps, ps, nb, st);
        } else {
            launch_forces_mixed<false>(sys, A, dps, ps, nb, st);
        }
    }
    MDG_LAUNCHED(ctx);
    if (stage == 1 && th) return launch_thermostat(sys, th, precision);
    return MDG_OK;
}

int launch_virials(mdg_system* sys, const PotSet* dps, const PotSet& ps) {
    mdg_ctx* ctx = sys->ctx;
    if (sys->n == 0) return MDG_OK;
    FArgs A = force_args(sys);
    int nb = nblk(sys->n);
    if (sys->half) {
        // accumulates onto the outputs: cleared first, as prepare leaves them
        int rc = launch_zero_meas(sys);
        if (rc) return rc;
        if (ps.multi) k_virials64<true, true><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
        else k_virials64<false, true><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
    } else {
        if (ps.multi) k_virials64<true, false><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
        else k_virials64<false, false><<<nb, kBlock, 0, ctx->stream>>>(A, dps);
    }
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

// ---------------------------------------------------------------------------
// Potential::value and EAM::embeddingEnergy on arrays (the analysis calls of
// python/mdcraft/solver/potential/_potential.cxx:88-168): the FP64 bodies of
// the force kernels. value: EAM.cxx:141-174 and pair.cxx:81-114 (V(r)/2r
// from the Vpar spline, 0 past the table, no cutoff test), LJs.cxx:61-71;
// LJsCut keeps Base::value (base.cxx:19): 0.
// ---------------------------------------------------------------------------

__global__ void k_pot_values(PotParams P, int n, const double* __restrict__ r2, double* __restrict__ u) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double e = 0.0;
    if (P.type == POT_EAM) eam_ff64(P, r2[i], 0.0, &e);
    else if (P.type == POT_TAB) tab_ff64(P, r2[i], &e);
    else if (P.type == POT_LJS) ljs_ff64(P, r2[i], &e);
    u[i] = e;
}

__global__ void k_pot_embedding(PotParams P, int n, const double* __restrict__ rho, double* __restrict__ F,
                                double* __restrict__ dF, DevStatus* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double EF = 0.0, d = 0.0;
    eam_embed64(P, rho[i], &EF, &d, st);
    F[i] = EF;
    dF[i] = d;
}

// ---- Potential::force / virial / density of one atom over an explicit list
// (the per-atom overloads of potential/base.h: LJs-cut.cxx:22-131,
// EAM.cxx:306-354, 465-497, 541-560). One thread walks the list in the
// reference's order with its FP64 arithmetic; recs[0] is the atom and
// slots[k] the record of list entry k. LJsCut with a half list pushes each
// pair's force, energy and virial onto the neighbour too; EAM ignores the
// half flag, as the reference does.
__global__ void k_pot_atom(PotParams P, int what, mdg_atom* recs, const uint32_t* __restrict__ slots, int count,
                           int half, DevStatus* st) {
    if (threadIdx.x != 0 || blockIdx.x != 0 || count == 0) return;
    mdg_atom& a = recs[0];
    const double x = a.r[0], y = a.r[1], z = a.r[2];
    if (P.type == POT_LJCUT) {
        double fx = 0.0, fy = 0.0, fz = 0.0;
        double Vxx = 0.0, Vyy = 0.0, Vzz = 0.0, Vxy = 0.0, Vxz = 0.0, Vyz = 0.0;
        for (int k = 0; k < count; ++k) {
            mdg_atom& nb = recs[slots[k]];
            const double dx = nb.r[0] - x, dy = nb.r[1] - y, dz = nb.r[2] - z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > P.R2cut || r2 < 1e-15) continue;
            const double pref = lj_pref64(P, r2);
            if (what == MDG_ATOM_FORCE) {
                fx += dx * pref;
                fy += dy * pref;
                fz += dz * pref;
                if (half) {
                    nb.f[0] -= dx * pref;
                    nb.f[1] -= dy * pref;
                    nb.f[2] -= dz * pref;
                }
            } else if (what == MDG_ATOM_VIRIAL) {
                const double ff[3] = {pref * dx, pref * dy, pref * dz}, d[3] = {dx, dy, dz};
                Vxx += ff[0] * dx;
                Vyy += ff[1] * dy;
                Vzz += ff[2] * dz;
                Vxy += ff[0] * dy;
                Vxz += ff[0] * dz;
                Vyz += ff[1] * dz;
                const double r2inv = 1.0 / r2;
                const double tmp = P.s6 * (r2inv * r2inv * r2inv);
                const double e = 0.5 * 4 * P.a * tmp * (tmp - 1);
                a.Ep += e;
                if (half) {
                    for (int c = 0; c < 3; ++c)
                        for (int r = 0; r < 3; ++r) nb.V[r + 3 * c] += 0.5 * (ff[r] * d[c]);
                    nb.Ep += e;
                }
            }
        }
        if (what == MDG_ATOM_FORCE) {
            a.f[0] += fx;
            a.f[1] += fy;
            a.f[2] += fz;
        } else if (what == MDG_ATOM_VIRIAL) {
            const double M[9] = {Vxx, Vxy, Vxz, Vxy, Vyy, Vyz, Vxz, Vyz, Vzz};
            for (int q = 0; q < 9; ++q) a.V[q] += 0.5 * M[q];
        }
        return;
    }
    if (P.type != POT_EAM) return;
    if (what == MDG_ATOM_DENSITY) {
        double sd = 0.0;
        for (int k = 0; k < count; ++k) {
            const mdg_atom& nb = recs[slots[k]];
            const double dx = nb.r[0] - x, dy = nb.r[1] - y, dz = nb.r[2] - z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > P.R2cut || r2 < 1e-15) continue;
            sd = sd + eam_rho64(P, sqrt(r2));
        }
        a.nc += sd;
        return;
    }
    // force and virial: F' of every listed neighbour's density and the atom's own
    double EFs = 0.0, dFs = 0.0;
    eam_embed64(P, a.nc, &EFs, &dFs, st);
    double F[3] = {0.0, 0.0, 0.0}, M[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Ep = 0.0;
    for (int k = 0; k < count; ++k) {
        const mdg_atom& nb = recs[slots[k]];
        double EFj = 0.0, dFj = 0.0;
        eam_embed64(P, nb.nc, &EFj, &dFj, st);
        const double d[3] = {nb.r[0] - x, nb.r[1] - y, nb.r[2] - z};
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 > P.R2cut || r2 < 1e-15) continue;
        double e = 0.0;
        const double FF = eam_ff64(P, r2, dFj + dFs, &e);
        if (what == MDG_ATOM_FORCE) {
            for (int q = 0; q < 3; ++q) F[q] += FF * d[q];
        } else {
            const double h = 0.5 * FF;
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r) M[r + 3 * c] += h * d[r] * d[c];
            Ep += e;
        }
    }
    if (what == MDG_ATOM_FORCE) {
        for (int q = 0; q < 3; ++q) a.f[q] += F[q];
    } else {
        a.Em = EFs;
        for (int q = 0; q < 9; ++q) a.V[q] += M[q];
        a.Ep += Ep;
    }
}

int pot_atom(const PotParams& P, int what, mdg_atom* recs_host, size_t nrec, const uint32_t* slots_host,
             size_t count, int half, cudaStream_t st, uint32_t* flags) {
    mdg_atom* d = nullptr;
    uint32_t* ds = nullptr;
    DevStatus* dst = nullptr;
    int rc = MDG_OK;
    cudaError_t e = cudaMalloc(&d, nrec * sizeof(mdg_atom));
    if (e == cudaSuccess) e = cudaMalloc(&ds, std::max<size_t>(count, 1) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMemsetAsync(dst, 0, sizeof(DevStatus), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, recs_host, nrec * sizeof(mdg_atom), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && count)
        e = cudaMemcpyAsync(ds, slots_host, count * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_pot_atom<<<1, 32, 0, st>>>(P, what, d, ds, (int)count, half, dst);
        e = cudaGetLastError();
    }
    DevStatus hs;
    memset(&hs, 0, sizeof(hs));
    if (e == cudaSuccess) e = cudaMemcpyAsync(recs_host, d, nrec * sizeof(mdg_atom), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "per-atom potential evaluation");
    if (flags) *flags = hs.flags;
    cudaFree(dst);
    cudaFree(ds);
    cudaFree(d);
    return rc;
}

// what = 0: u[k] = value(x[k]); what = 1: F, dF of density x[k]. Host arrays
// in and out through one device scratch block; waits on `st`.
int pot_eval(const PotParams& P, int what, const double* x, size_t n, double* out0, double* out1,
             cudaStream_t st) {
    if (n == 0) return MDG_OK;
    if (n > (size_t)INT32_MAX) {
        set_error("too many values in one call");
        return MDG_ERR_INVALID;
    }
    double* d = nullptr;
    DevStatus* ds = nullptr;
    MDG_CUDA(cudaMalloc(&d, 3 * n * sizeof(double)));
    int rc = MDG_OK;
    cudaError_t e = cudaMalloc(&ds, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMemsetAsync(ds, 0, sizeof(DevStatus), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, x, n * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        if (what == 0) k_pot_values<<<nblk(n), kBlock, 0, st>>>(P, (int)n, d, d + n);
        else k_pot_embedding<<<nblk(n), kBlock, 0, st>>>(P, (int)n, d, d + n, d + 2 * n, ds);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out0, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && out1)
        e = cudaMemcpyAsync(out1, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_status(e, "potential evaluation");
    cudaFree(ds);
    cudaFree(d);
    return rc;
}

}  // namespace mdg
