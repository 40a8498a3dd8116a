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
    float4* pos32;
    const float4* o0;
    const float* trig;
    DevStatus* st;
};

__device__ __forceinline__ void flag_need(bool need, DevStatus* st) {
    unsigned b = __ballot_sync(__activemask(), need);
    if (b && (threadIdx.x & 31) == (__ffs(b) - 1)) atomicOr(&st->need_rebuild, 1u);
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

// Mixed form: kick + drift, cell-offset refresh, half-skin test.
__device__ __forceinline__ bool drift_mixed_one(const IArgs& A, int i) {
    bool need = false;
    {
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
        float o[3] = {(float)(r[0] - A.Rx[i]), (float)(r[1] - A.Ry[i]), (float)(r[2] - A.Rz[i])};
        A.pos32[i] = make_float4(o[0], o[1], o[2], 0.0f);
        float4 q = A.o0[i];
        float dx = o[0] - q.x, dy = o[1] - q.y, dz = o[2] - q.z;
        float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        need = d2 > A.trig[i];
    }
    return need;
}

__device__ __forceinline__ void kick_mixed_one(const IArgs& A, int i) {
    if (A.tag[i] == 0) return;
    float hm = (0.5f * (float)A.dt) * __frcp_rn((float)A.m[i]);
    A.vx[i] += (double)(A.gx[i] * hm);
    A.vy[i] += (double)(A.gy[i] * hm);
    A.vz[i] += (double)(A.gz[i] * hm);
}

// Half-skin threshold per atom for the mixed test: (skin/2)^2 shrunk by
// 1e-6 so that FP32 rounding can only trigger a rebuild early.
__device__ __forceinline__ void trig_one(int i, const double* __restrict__ saved_rns,
                                         const double* __restrict__ saved_rcut, float* __restrict__ trig) {
    double skin = saved_rns[i] - saved_rcut[i];
    trig[i] = skin <= 0.0 ? -1.0f : (float)(0.25 * skin * skin * (1.0 - 1e-6));
}

}  // namespace mdg

struct mdg_system;

namespace mdg {
// Argument block of a system's integrator passes (integrate.cu).
IArgs integrator_args(mdg_system* sys, double dt);
}  // namespace mdg
