// integrate_dev.cuh — per-atom bodies of the velocity-Verlet halves, the
// rebuild test and its threshold, shared by the per-stage kernels
// (integrate.cu) and the fused per-system loop (solo.cu).
//
// Verlet::step_one_coords / step_one_velocities
// (mdcraft/solver/stepper/verlet.cxx:71-85) and VerletList::decide
// (mdcraft/neibs/verlet-list.cxx:127-155).
#pragma once

#include <cuda_runtime.h>

#include "mdg_internal.cuh"

namespace mdg {

struct IArgs {
    int n;
    double dt;
    double *rx, *ry, *rz, *vx, *vy, *vz;
    const double *fx, *fy, *fz;
    const float *gx, *gy, *gz;
    const double* m;
    const uint16_t* tag;
    const uint16_t* kind;  // w of the fixed-point offsets (pos32): the atom's kind
    double* rcut;
    const double* rns;
    const uint32_t* uid;
    const double *r0x, *r0y, *r0z, *saved_rcut, *saved_rns;
    const uint32_t* saved_uid;
    uint8_t* bc;
    double pot_rcut;  // < 0: leave rcut (Multi::prepare_one does not set it)
    int periodic_boundary;
    double bmin[3], bmax[3], L[3];
    int periodic[3];
    // mixed
    const double *Rx, *Ry, *Rz;
    int4* pos32;
    const int4* q0;      // fixed-point offsets at the last rebuild
    double inv_u[3];     // fixed-point offset units per axis (GridParams::inv_u)
    float uf[3];         // their lengths in FP32 (cs / 2^29)
    const float2* trig;  // (skin/2)^2 of the last rebuild (-1 when skin <= 0) and its band (trig_one)
    DevStatus* st;
};

__device__ __forceinline__ void flag_need(bool need, DevStatus* st) {
    unsigned b = __ballot_sync(__activemask(), need);
    if (b && (threadIdx.x & 31) == (__ffs(b) - 1)) atomicOr(&st->need_rebuild, 1u);
}

__device__ __forceinline__ void flag_need_next(bool need, DevStatus* st) {
    unsigned b = __ballot_sync(__activemask(), need);
    if (b && (threadIdx.x & 31) == (__ffs(b) - 1)) atomicOr(&st->need_next, 1u);
}

// VerletList::decide per atom (verlet-list.cxx:135-154), exact FP64.
__device__ __forceinline__ bool decide_one(const IArgs& A, int i, double x, double y, double z) {
    if (A.uid[i] != A.saved_uid[i] || A.rcut[i] != A.saved_rcut[i] || A.rns[i] != A.saved_rns[i]) return true;
    double skin = dsub(A.saved_rns[i], A.saved_rcut[i]);
    if (skin <= 0.0) return true;
    double dx = shortest1(dsub(x, A.r0x[i]), A.L[0], A.periodic[0]);
    double dy = shortest1(dsub(y, A.r0y[i]), A.L[1], A.periodic[1]);
    double dz = shortest1(dsub(z, A.r0z[i]), A.L[2], A.periodic[2]);
    double trigger2 = dmul(dmul(0.25, skin), skin);
    return sq3_exact(dx, dy, dz) > trigger2;
}

// step_one_coords + prepare + decide, FP64 form (drift = 0: the prepare
// part alone, Pair::prepare called on its own).
__device__ __forceinline__ bool drift64_one(const IArgs& A, int i, int drift, int check) {
    bool need = false;
    {
        double r[3] = {A.rx[i], A.ry[i], A.rz[i]};
        uint16_t tg = A.tag[i];
        if (drift && tg != 0) {
            double f[3] = {A.fx[i], A.fy[i], A.fz[i]};
            double v[3] = {A.vx[i], A.vy[i], A.vz[i]};
            double m = A.m[i];
            for (int k = 0; k < 3; ++k) {
                double a = __ddiv_rn(f[k], m);
                v[k] = dadd(v[k], dmul(dmul(a, A.dt), 0.5));
                r[k] = dadd(r[k], dmul(v[k], A.dt));
            }
            A.rx[i] = r[0]; A.ry[i] = r[1]; A.rz[i] = r[2];
            A.vx[i] = v[0]; A.vy[i] = v[1]; A.vz[i] = v[2];
        }
        if (tg != 0 && A.pot_rcut >= 0.0) A.rcut[i] = A.pot_rcut;
        uint8_t bc = 0;
        if (A.periodic_boundary && tg != 0) {
            double rn = A.rns[i];
            for (int a = 0; a < 3; ++a) {
                if (!A.periodic[a]) continue;
                double d0 = fabs(dsub(r[a], A.bmin[a])), d1 = fabs(dsub(r[a], A.bmax[a]));
                if ((d0 < d1 ? d0 : d1) < rn) bc = 1;
            }
        }
        A.bc[i] = bc;
        if (check) need = decide_one(A, i, r[0], r[1], r[2]);
    }
    return need;
}

// Mixed form: kick + drift, cell-offset refresh, and the half-skin test of
// VerletList::decide (verlet-list.cxx:135-154) with the FP64 result: the
// displacement since the rebuild is first taken from the fixed-point offsets
// (q - q0, exact up to one offset unit per axis) in FP32; only an atom whose
// estimate lies within the proven error band around (skin/2)^2 (trig_one;
// about 1e-5 of it) is tested again with the reference's FP64 arithmetic, so
// every decision equals decide_one's on the same positions. (The size, uid,
// rcut and rns comparisons of decide cannot change inside the step loop: the
// drift does not touch those fields, and a host-side change marks the list
// stale.)
// The offsets refresh and the rebuild test of drift_mixed_one, for the
// atom's position r after its drift.
__device__ __forceinline__ bool offsets_check_mixed(const IArgs& A, int i, const double r[3]) {
    const int4 q = make_int4(off_encode(r[0] - __ldcs(A.Rx + i), A.inv_u[0]),
                             off_encode(r[1] - __ldcs(A.Ry + i), A.inv_u[1]),
                             off_encode(r[2] - __ldcs(A.Rz + i), A.inv_u[2]), __ldcs(A.kind + i) & 3);
    A.pos32[i] = q;
    const int4 p = __ldcs(A.q0 + i);
    const float dx = __int2float_rn((int)((uint32_t)q.x - (uint32_t)p.x)) * A.uf[0];
    const float dy = __int2float_rn((int)((uint32_t)q.y - (uint32_t)p.y)) * A.uf[1];
    const float dz = __int2float_rn((int)((uint32_t)q.z - (uint32_t)p.z)) * A.uf[2];
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float2 tb = __ldcs(A.trig + i);
    if (d2 > tb.x + tb.y) return true;
    if (d2 < tb.x - tb.y) return false;
    double skin = dsub(A.saved_rns[i], A.saved_rcut[i]);
    double ex = shortest1(dsub(r[0], A.r0x[i]), A.L[0], A.periodic[0]);
    double ey = shortest1(dsub(r[1], A.r0y[i]), A.L[1], A.periodic[1]);
    double ez = shortest1(dsub(r[2], A.r0z[i]), A.L[2], A.periodic[2]);
    return skin <= 0.0 || sq3_exact(ex, ey, ez) > dmul(dmul(0.25, skin), skin);
}

__device__ __forceinline__ bool drift_mixed_one(const IArgs& A, int i) {
    double r[3] = {A.rx[i], A.ry[i], A.rz[i]};
    if (A.tag[i] != 0) {
        float hm = (0.5f * (float)A.dt) * __frcp_rn((float)A.m[i]);
        float g[3] = {A.gx[i], A.gy[i], A.gz[i]};
        double* v[3] = {A.vx, A.vy, A.vz};
        for (int k = 0; k < 3; ++k) {
            double vk = v[k][i] + (double)(g[k] * hm);
            v[k][i] = vk;
            r[k] = fma(vk, A.dt, r[k]);
        }
        A.rx[i] = r[0]; A.ry[i] = r[1]; A.rz[i] = r[2];
    }
    return offsets_check_mixed(A, i, r);
}

// Per-atom fields read once per step (cell centres, rebuild-time offsets
// and thresholds, mass, position, velocity) are loaded cache-streaming
// (evict-first), so that they do not displace the neighbour records and
// table rows the force pass gathers from L1.
// The end of a mixed step's force pass when the next step starts in it:
// the FP32 force stored, this step's second half-kick, then the next
// step's first half-kick and drift, offsets refresh and rebuild test —
// kick_mixed_one followed by drift_mixed_one, operation for operation
// (the same FP32 increment added to v twice, r advanced by fma(v, dt, r)).
// Returns the rebuild test of the new position.
__device__ __forceinline__ bool kick_drift_mixed(const IArgs& A, float* gx, float* gy, float* gz, int i, float fx,
                                                 float fy, float fz) {
    gx[i] = fx;
    gy[i] = fy;
    gz[i] = fz;
    const float hm = (0.5f * (float)A.dt) * __frcp_rn((float)__ldcs(A.m + i));
    const float g[3] = {fx, fy, fz};
    double* v[3] = {A.vx, A.vy, A.vz};
    double r[3] = {__ldcs(A.rx + i), __ldcs(A.ry + i), __ldcs(A.rz + i)};
    for (int k = 0; k < 3; ++k) {
        double vk = __ldcs(v[k] + i) + (double)(g[k] * hm);  // second half-kick of this step
        vk = vk + (double)(g[k] * hm);               // first half-kick of the next
        v[k][i] = vk;
        r[k] = fma(vk, A.dt, r[k]);
    }
    A.rx[i] = r[0]; A.ry[i] = r[1]; A.rz[i] = r[2];
    return offsets_check_mixed(A, i, r);
}

__device__ __forceinline__ void kick_mixed_one(const IArgs& A, int i) {
    if (A.tag[i] == 0) return;
    float hm = (0.5f * (float)A.dt) * __frcp_rn((float)A.m[i]);
    A.vx[i] += (double)(A.gx[i] * hm);
    A.vy[i] += (double)(A.gy[i] * hm);
    A.vz[i] += (double)(A.gz[i] * hm);
}

// Half-skin threshold per atom for the mixed form's test: (0.25 skin) skin
// as decide_one computes it (-1, always rebuild, when skin <= 0), and the
// band within which the FP32 estimate of drift_mixed_one cannot decide. Its
// error is at most sqrt(3) u per axis from the offset quantisation (u the
// largest offset unit), i.e. 2 sqrt(3) |d| u + 3 u^2 in d^2, plus ~1e-6
// relative from the FP32 arithmetic; the band, 1e-5 of the threshold +
// 4 sqrt(threshold) u + 4 u^2, covers both. The threshold is FP64 (as
// decide_one's) rounded to FP32; the band, a bound with 15% or more to
// spare in each term, is evaluated in FP32 (FP64 square roots are slow).
__device__ __forceinline__ void trig_one(int i, const double* __restrict__ saved_rns,
                                         const double* __restrict__ saved_rcut, const GridParams& g,
                                         float2* __restrict__ trig) {
    double skin = dsub(saved_rns[i], saved_rcut[i]);
    if (skin <= 0.0) {
        trig[i] = make_float2(-1.0f, 0.0f);
        return;
    }
    const float t = (float)dmul(dmul(0.25, skin), skin);
    const float u = fmaxf(g.csf[0], fmaxf(g.csf[1], g.csf[2])) * (1.0f / (float)kOffUnits);
    trig[i] = make_float2(t, fmaf(1e-5f, t, fmaf(4.0f * sqrtf(t), u, 4.0f * u * u)));
}

}  // namespace mdg

struct mdg_system;

namespace mdg {
// Argument block of a system's integrator passes (integrate.cu).
IArgs integrator_args(mdg_system* sys, double dt);
}  // namespace mdg
