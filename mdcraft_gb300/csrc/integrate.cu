// integrate.cu — velocity-Verlet, Pair::prepare, the rebuild test, and FP64
// measurement reductions.
//
// FP64 form: Verlet::step_one_coords / step_one_velocities
// (mdcraft/solver/stepper/verlet.cxx:71-85) with the reference's operation
// order and no FMA contraction, fused with Single::prepare_one's rcut
// (single.cxx:38-53), Periodic::prepare_one's boundary flag
// (periodic.cxx:9-34) and VerletList::decide's test (verlet-list.cxx:127-155)
// on the new positions, so one pass per atom yields the step's drift and
// the rebuild flag.
//
// Mixed form: FP64 positions and velocities, velocity increments computed in
// FP32 from the FP32 forces, FP64 accumulation; the same pass refreshes the
// fixed-point cell-centred offsets used by the pair kernels and runs the
// half-skin test in FP64 on the new positions.
#include <cuda_runtime.h>

#include "mdg_host.h"
#include "integrate_dev.cuh"

namespace mdg {




// step_one_coords + prepare + decide (FP64 form). drift = 0 runs only the
// prepare + decide part (Pair::prepare called on its own).
__global__ void k_drift64(IArgs A, int drift, int check) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = i < A.n ? drift64_one(A, i, drift, check) : false;
    if (check) flag_need(need, A.st);
}

// VerletList::decide on its own (mdg_nlist_decide).
__global__ void k_decide(IArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = false;
    if (i < A.n) need = decide_one(A, i, A.rx[i], A.ry[i], A.rz[i]);
    flag_need(need, A.st);
}

// step_one_velocities (verlet.cxx:80-85), FP64 form.
__global__ void k_kick64(IArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n || A.tag[i] == 0) return;
    double m = A.m[i];
    double* v[3] = {A.vx, A.vy, A.vz};
    const double* f[3] = {A.fx, A.fy, A.fz};
    for (int k = 0; k < 3; ++k) {
        double a = __ddiv_rn(f[k][i], m);
        v[k][i] = dadd(v[k][i], dmul(dmul(a, 0.5), A.dt));
    }
}

// Mixed form: kick + drift, cell-offset refresh, half-skin test.
__global__ void k_drift_mixed(IArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = i < A.n ? drift_mixed_one(A, i) : false;
    flag_need(need, A.st);
}

// The mixed drift as its own pass inside the step loop's graph, where the
// force pass could not start the step (the first step, after a rebuild):
// skipped on the device when fewer than min_left steps remain or the
// rebuild before it outgrew its capacities.
__global__ void k_drift_mixed_guarded(IArgs A, const unsigned long long* __restrict__ left,
                                      unsigned long long min_left) {
    if (*left < min_left || (A.st->build_flags & FLAG_OVERFLOW)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool need = i < A.n ? drift_mixed_one(A, i) : false;
    flag_need(need, A.st);
}

__global__ void k_kick_mixed(IArgs A) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) kick_mixed_one(A, i);
}

// Half-skin threshold per atom for the mixed test (trig_one).
__global__ void k_trig(int n, const double* __restrict__ saved_rns, const double* __restrict__ saved_rcut,
                       const GridParams* __restrict__ gp, float2* __restrict__ trig) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) trig_one(i, saved_rns, saved_rcut, *gp, trig);
}

// Refresh of the fixed-point offsets from FP64 positions (after uploads).
__global__ void k_offsets(int n, const double* __restrict__ rx, const double* __restrict__ ry,
                          const double* __restrict__ rz, const double* __restrict__ Rx,
                          const double* __restrict__ Ry, const double* __restrict__ Rz, double ux, double uy,
                          double uz, int4* __restrict__ pos32, const uint16_t* __restrict__ kind) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos32[i] = make_int4(off_encode(rx[i] - Rx[i], ux), off_encode(ry[i] - Ry[i], uy), off_encode(rz[i] - Rz[i], uz),
                         kind[i] & 3);
}

// FP32 -> FP64 force copy after a mixed stage, so downloads and a later
// FP64 step see the mixed forces.
__global__ void k_forces_to64(int n, const float* __restrict__ gx, const float* __restrict__ gy,
                              const float* __restrict__ gz, const uint16_t* __restrict__ tag,
                              double* __restrict__ fx, double* __restrict__ fy, double* __restrict__ fz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || tag[i] == 0) return;
    fx[i] = gx[i];
    fy[i] = gy[i];
    fz[i] = gz[i];
}

__global__ void k_forces_to32(int n, const double* __restrict__ fx, const double* __restrict__ fy,
                              const double* __restrict__ fz, float* __restrict__ gx, float* __restrict__ gy,
                              float* __restrict__ gz) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    gx[i] = (float)fx[i];
    gy[i] = (float)fy[i];
    gz[i] = (float)fz[i];
}

// Pair::prepare's zeroing of the accumulators (single.cxx:38-53).
struct ZeroArgs {
    double *fx, *fy, *fz, *Ep, *Em, *nc;
    double* V[9];  // nine separate allocations
};

// Pair::prepare's resets for atoms with tag != 0: fields selected by
// `what` (ZERO_* bits).
enum : int { ZERO_F = 1, ZERO_EP_V = 2, ZERO_EM = 4, ZERO_NC = 8 };

__global__ void k_zero_outputs(int n, const uint16_t* __restrict__ tag, ZeroArgs Z, int what) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || tag[i] == 0) return;
    if (what & ZERO_F) { Z.fx[i] = 0.0; Z.fy[i] = 0.0; Z.fz[i] = 0.0; }
    if (what & ZERO_EP_V) {
        Z.Ep[i] = 0.0;
        for (int k = 0; k < 9; ++k) Z.V[k][i] = 0.0;
    }
    if (what & ZERO_EM) Z.Em[i] = 0.0;
    if (what & ZERO_NC) Z.nc[i] = 0.0;
}

// ---- FP64 reductions: measure_state (md_test_utils.h:214-239) --------------
struct MArgs {
    int n;
    const double *Ep, *Em, *V0, *V4, *V8, *m, *vx, *vy, *vz;
    double* part;
};

__device__ void block_sum(double* sh, double* vals, int nv) {
    int t = threadIdx.x;
    for (int k = 0; k < nv; ++k) sh[k * kBlock + t] = vals[k];
    __syncthreads();
    for (int s = kBlock / 2; s > 0; s >>= 1) {
        if (t < s)
            for (int k = 0; k < nv; ++k) sh[k * kBlock + t] += sh[k * kBlock + t + s];
        __syncthreads();
    }
}

__global__ void k_measure1(MArgs A) {
    __shared__ double sh[7 * kBlock];
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        v[0] += A.Ep[i];
        v[1] += A.Em[i];
        v[2] += A.V0[i] + A.V4[i] + A.V8[i];
        v[3] += A.m[i] * A.vx[i];
        v[4] += A.m[i] * A.vy[i];
        v[5] += A.m[i] * A.vz[i];
        v[6] += A.m[i];
    }
    block_sum(sh, v, 7);
    if (threadIdx.x < 7) A.part[blockIdx.x * 8 + threadIdx.x] = sh[threadIdx.x * kBlock];
}

__global__ void k_measure2(MArgs A, const double* __restrict__ com) {
    __shared__ double sh[kBlock];
    double ke = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double dx = A.vx[i] - com[0], dy = A.vy[i] - com[1], dz = A.vz[i] - com[2];
        ke += 0.5 * A.m[i] * (dx * dx + dy * dy + dz * dz);
    }
    double v[1] = {ke};
    block_sum(sh, v, 1);
    if (threadIdx.x == 0) A.part[blockIdx.x * 8 + 7] = sh[0];
}

__global__ void k_measure_final(const double* __restrict__ part, int nparts, int stage, double* __restrict__ out) {
    // one thread, fixed order: deterministic
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (stage == 1) {
        double s[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int b = 0; b < nparts; ++b)
            for (int k = 0; k < 7; ++k) s[k] += part[b * 8 + k];
        for (int k = 0; k < 7; ++k) out[k] = s[k];
        double tm = s[6];
        out[8] = tm > 0.0 ? s[3] / tm : 0.0;
        out[9] = tm > 0.0 ? s[4] / tm : 0.0;
        out[10] = tm > 0.0 ? s[5] / tm : 0.0;
    } else {
        double ke = 0.0;
        for (int b = 0; b < nparts; ++b) ke += part[b * 8 + 7];
        out[7] = ke;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

IArgs integrator_args(mdg_system* sys, double dt) {
    IArgs A;
    memset(&A, 0, sizeof(A));
    int c = sys->cur;
    A.n = (int)sys->n;
    A.dt = dt;
    A.rx = sys->f64[RX][c]; A.ry = sys->f64[RY][c]; A.rz = sys->f64[RZ][c];
    A.vx = sys->f64[VX][c]; A.vy = sys->f64[VY][c]; A.vz = sys->f64[VZ][c];
    A.fx = sys->f64[FX][c]; A.fy = sys->f64[FY][c]; A.fz = sys->f64[FZ][c];
    A.gx = sys->f32[0][c]; A.gy = sys->f32[1][c]; A.gz = sys->f32[2][c];
    A.m = sys->f64[MASS][c];
    A.tag = sys->u16[TAG][c];
    A.kind = sys->u16[KIND][c];
    A.rcut = sys->f64[RCUT][c];
    A.rns = sys->f64[RNS][c];
    A.uid = sys->u32[UID][c];
    A.r0x = sys->r0[0]; A.r0y = sys->r0[1]; A.r0z = sys->r0[2];
    A.saved_rcut = sys->saved_rcut;
    A.saved_rns = sys->saved_rns;
    A.saved_uid = sys->saved_uid;
    A.bc = sys->bc;
    A.pot_rcut = -1.0;
    for (int a = 0; a < 3; ++a) {
        A.bmin[a] = sys->dom.bmin[a];
        A.bmax[a] = sys->dom.bmax[a];
        A.L[a] = sys->dom.bmax[a] - sys->dom.bmin[a];
        A.periodic[a] = sys->dom.periodic[a] ? 1 : 0;
    }
    A.Rx = sys->Rc[0]; A.Ry = sys->Rc[1]; A.Rz = sys->Rc[2];
    A.pos32 = sys->pos32;
    A.q0 = sys->q0;
    for (int a = 0; a < 3; ++a) {
        A.inv_u[a] = sys->grid.inv_u[a];
        A.uf[a] = (float)(sys->grid.cs[a] / kOffUnits);
    }
    A.trig = sys->trig32;
    A.st = sys->dstat;
    return A;
}

int launch_drift(mdg_system* sys, double dt, int precision, double pot_rcut, int periodic_boundary,
                 int drift, int check) {
    if (sys->n == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    IArgs A = integrator_args(sys, dt);
    A.pot_rcut = pot_rcut;
    A.periodic_boundary = periodic_boundary;
    if (precision == MDG_PREC_MIXED && drift) k_drift_mixed<<<nblk(sys->n), kBlock, 0, ctx->stream>>>(A);
    else k_drift64<<<nblk(sys->n), kBlock, 0, ctx->stream>>>(A, drift, check);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

int launch_drift_guarded(mdg_system* sys, double dt, const unsigned long long* left, unsigned long long min_left) {
    if (sys->n == 0) return MDG_OK;
    IArgs A = integrator_args(sys, dt);
    k_drift_mixed_guarded<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>(A, left, min_left);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

int launch_decide(mdg_system* sys) {
    if (sys->n == 0) return MDG_OK;
    IArgs A = integrator_args(sys, 0.0);
    k_decide<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>(A);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

int launch_kick(mdg_system* sys, double dt, int precision) {
    if (sys->n == 0) return MDG_OK;
    mdg_ctx* ctx = sys->ctx;
    IArgs A = integrator_args(sys, dt);
    if (precision == MDG_PREC_MIXED) k_kick_mixed<<<nblk(sys->n), kBlock, 0, ctx->stream>>>(A);
    else k_kick64<<<nblk(sys->n), kBlock, 0, ctx->stream>>>(A);
    MDG_LAUNCHED(ctx);
    return MDG_OK;
}

int launch_trig(mdg_system* sys) {
    if (sys->n == 0) return MDG_OK;
    k_trig<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>((int)sys->n, sys->saved_rns, sys->saved_rcut,
                                                          sys->dgrid, sys->trig32);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

int launch_offsets(mdg_system* sys) {
    if (sys->n == 0) return MDG_OK;
    int c = sys->cur;
    k_offsets<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>((int)sys->n, sys->f64[RX][c], sys->f64[RY][c],
                                                             sys->f64[RZ][c], sys->Rc[0], sys->Rc[1], sys->Rc[2],
                                                             sys->grid.inv_u[0], sys->grid.inv_u[1],
                                                             sys->grid.inv_u[2], sys->pos32, sys->u16[KIND][c]);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

int launch_force_copy(mdg_system* sys, int to64) {
    if (sys->n == 0) return MDG_OK;
    int c = sys->cur;
    if (to64)
        k_forces_to64<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>(
            (int)sys->n, sys->f32[0][c], sys->f32[1][c], sys->f32[2][c], sys->u16[TAG][c], sys->f64[FX][c],
            sys->f64[FY][c], sys->f64[FZ][c]);
    else
        k_forces_to32<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>(
            (int)sys->n, sys->f64[FX][c], sys->f64[FY][c], sys->f64[FZ][c], sys->f32[0][c], sys->f32[1][c],
            sys->f32[2][c]);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

static int launch_zero_fields(mdg_system* sys, int what);

int launch_zero(mdg_system* sys, int eam) {
    if (sys->n == 0) return MDG_OK;
    if (eam) sys->fp_ok = 0;  // nc cleared
    // prepare clears the measurement outputs as well
    sys->stale_out &= eam ? 0 : ~STALE_EP_V;
    return launch_zero_fields(sys, ZERO_F | ZERO_EP_V | (eam ? ZERO_EM | ZERO_NC : 0));
}

// The measurement outputs a step's prepare would have cleared, cleared now
// that something reads them (they are not rewritten every step).
int settle_outputs(mdg_system* sys) {
    if (sys->n == 0 || !sys->stale_out) return MDG_OK;
    const int what = ((sys->stale_out & STALE_EP_V) ? ZERO_EP_V : 0) | ((sys->stale_out & STALE_EM) ? ZERO_EM : 0);
    sys->stale_out = 0;
    return launch_zero_fields(sys, what);
}

int launch_zero_meas(mdg_system* sys) {
    if (sys->n == 0) return MDG_OK;
    return launch_zero_fields(sys, ZERO_EP_V);
}

static int launch_zero_fields(mdg_system* sys, int what) {
    int c = sys->cur;
    ZeroArgs Z;
    Z.fx = sys->f64[FX][c];
    Z.fy = sys->f64[FY][c];
    Z.fz = sys->f64[FZ][c];
    Z.Ep = sys->f64[EP][c];
    Z.Em = sys->f64[EM][c];
    Z.nc = sys->f64[NC][c];
    for (int k = 0; k < 9; ++k) Z.V[k] = sys->f64[V0 + k][c];
    k_zero_outputs<<<nblk(sys->n), kBlock, 0, sys->ctx->stream>>>((int)sys->n, sys->u16[TAG][c], Z, what);
    MDG_LAUNCHED(sys->ctx);
    return MDG_OK;
}

int launch_measure(mdg_system* sys, double out[11]) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    int c = sys->cur;
    MArgs A;
    A.n = (int)sys->n;
    A.Ep = sys->f64[EP][c];
    A.Em = sys->f64[EM][c];
    A.V0 = sys->f64[V0][c];
    A.V4 = sys->f64[V4][c];
    A.V8 = sys->f64[V8][c];
    A.m = sys->f64[MASS][c];
    A.vx = sys->f64[VX][c];
    A.vy = sys->f64[VY][c];
    A.vz = sys->f64[VZ][c];
    int nparts = std::min(std::max(nblk(sys->n), 1), 4 * std::max(ctx->num_sms, 1));
    if ((size_t)nparts > sys->part_cap) {
        sys_free(sys, sys->part, sys->part_cap * 8 * sizeof(double));
        sys->part = nullptr;
        sys->part_cap = 0;
        int rc = sys_malloc(sys, (void**)&sys->part, (size_t)nparts * 8 * sizeof(double));
        if (rc) return rc;
        sys->part_cap = nparts;
    }
    A.part = sys->part;
    k_measure1<<<nparts, kBlock, 0, st>>>(A);
    MDG_LAUNCHED(ctx);
    k_measure_final<<<1, 32, 0, st>>>(sys->part, nparts, 1, sys->red);
    MDG_LAUNCHED(ctx);
    k_measure2<<<nparts, kBlock, 0, st>>>(A, sys->red + 8);
    MDG_LAUNCHED(ctx);
    k_measure_final<<<1, 32, 0, st>>>(sys->part, nparts, 2, sys->red);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(sys->hred, sys->red, 11 * sizeof(double), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 11; ++k) out[k] = sys->hred[k];
    return MDG_OK;
}

}  // namespace mdg
