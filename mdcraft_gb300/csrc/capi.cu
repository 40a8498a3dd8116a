// capi.cu — the extern "C" entry points of include/mdg.h.
//
// Host orchestration only: object lifetimes, host<->device transfers in the
// caller's atom order, spline set-up of EAM tables, the stage sequence of
// Single / Multi (mdcraft/solver/{single,multi}.cxx) and the Verlet step
// loop (mdcraft/solver/stepper/verlet.cxx:36-48). All arithmetic on atoms
// happens in the kernels of nlist.cu, forces.cu and integrate.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "mdg_host.h"

namespace mdg {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int cuda_status(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return MDG_ERR_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return MDG_ERR_NODEV;
    return MDG_ERR_CUDA;
}

int launch_stage(mdg_system* sys, const PotSet* dps, const PotSet& ps, int precision, int stage,
                 const ThermoDev* th, double kick_dt = 0.0);
int launch_virials(mdg_system* sys, const PotSet* dps, const PotSet& ps);
int launch_drift(mdg_system* sys, double dt, int precision, double pot_rcut, int periodic_boundary, int drift,
                 int check);
int launch_kick(mdg_system* sys, double dt, int precision);
int launch_forces_step(mdg_system* sys, const PotSet* dps, const PotSet& ps, double dt,
                       const unsigned long long* left);
int launch_drift_guarded(mdg_system* sys, double dt, const unsigned long long* left, unsigned long long min_left);
int ensure_cutbits(mdg_system* sys);
int launch_density_rec(mdg_system* sys, const PotSet* dps, const PotSet& ps);
int launch_decide(mdg_system* sys);
int launch_trig(mdg_system* sys);
int launch_offsets(mdg_system* sys);
int launch_force_copy(mdg_system* sys, int to64);
int launch_zero(mdg_system* sys, int eam);
int launch_measure(mdg_system* sys, double out[11]);

// ---------------------------------------------------------------------------
// transfers between the caller's order and the device slot order
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int b = kBlock) { return (int)((n + b - 1) / b); }

struct XferArgs {
    int n;
    const uint32_t* slot_of;
    double* f64[NF64];
    float* f32[3];
    uint32_t* u32[NU32];
    uint16_t* u16[NU16];
};

static XferArgs xfer_args(mdg_system* sys) {
    XferArgs X;
    memset(&X, 0, sizeof(X));
    int c = sys->cur;
    X.n = (int)sys->n;
    X.slot_of = sys->slot_of;
    for (int f = 0; f < NF64; ++f) X.f64[f] = sys->f64[f][c];
    for (int f = 0; f < 3; ++f) X.f32[f] = sys->f32[f][c];
    for (int f = 0; f < NU32; ++f) X.u32[f] = sys->u32[f][c];
    for (int f = 0; f < NU16; ++f) X.u16[f] = sys->u16[f][c];
    return X;
}

// 208-byte Atom records (caller order) -> SoA slots.
__global__ void k_atoms_in(XferArgs X, const mdg_atom* __restrict__ in) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= X.n) return;
    const mdg_atom& a = in[k];
    uint32_t s = X.slot_of[k];
    for (int c = 0; c < 3; ++c) {
        X.f64[RX + c][s] = a.r[c];
        X.f64[VX + c][s] = a.v[c];
        X.f64[FX + c][s] = a.f[c];
        X.f32[c][s] = (float)a.f[c];
    }
    X.f64[MASS][s] = a.m;
    X.f64[RCUT][s] = a.rcut;
    X.f64[RNS][s] = a.rns;
    X.f64[EP][s] = a.Ep;
    X.f64[EM][s] = a.Em;
    X.f64[NC][s] = a.nc;
    for (int q = 0; q < 9; ++q) X.f64[V0 + q][s] = a.V[q];
    X.u32[UID][s] = a.uid;
    X.u16[KIND][s] = a.kind;
    X.u16[TAG][s] = a.tag;
}

__global__ void k_atoms_out(XferArgs X, const uint8_t* __restrict__ bc, mdg_atom* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= X.n) return;
    mdg_atom& a = out[k];
    uint32_t s = X.slot_of[k];
    for (int c = 0; c < 3; ++c) {
        a.r[c] = X.f64[RX + c][s];
        a.v[c] = X.f64[VX + c][s];
        a.f[c] = X.f64[FX + c][s];
    }
    a.m = X.f64[MASS][s];
    a.rcut = X.f64[RCUT][s];
    a.rns = X.f64[RNS][s];
    a.Ep = X.f64[EP][s];
    a.Em = X.f64[EM][s];
    a.nc = X.f64[NC][s];
    for (int q = 0; q < 9; ++q) a.V[q] = X.f64[V0 + q][s];
    a.uid = X.u32[UID][s];
    a.kind = X.u16[KIND][s];
    a.tag = X.u16[TAG][s];
    a.bc = bc[s];
    a._pad[0] = a._pad[1] = a._pad[2] = 0;
}

// xyz triples (caller order) <-> three SoA fields.
__global__ void k_vec_in(int n, const uint32_t* __restrict__ slot_of, const double* __restrict__ in, double* x,
                         double* y, double* z) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s = slot_of[k];
    x[s] = in[3 * k];
    y[s] = in[3 * k + 1];
    z[s] = in[3 * k + 2];
}

__global__ void k_vec_out(int n, const uint32_t* __restrict__ slot_of, const double* x, const double* y,
                          const double* z, double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s = slot_of[k];
    out[3 * k] = x[s];
    out[3 * k + 1] = y[s];
    out[3 * k + 2] = z[s];
}

// Forces of the mixed form (FP32) into caller-order doubles.
__global__ void k_vec_out32(int n, const uint32_t* __restrict__ slot_of, const float* x, const float* y,
                            const float* z, double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s = slot_of[k];
    out[3 * k] = (double)x[s];
    out[3 * k + 1] = (double)y[s];
    out[3 * k + 2] = (double)z[s];
}

__global__ void k_iota(int n, uint32_t* a, uint32_t* b) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        a[k] = (uint32_t)k;
        b[k] = (uint32_t)k;
    }
}

cudaEvent_t timer_begin(mdg_ctx* ctx) {
    if (!ctx->timing) return nullptr;
    cudaEvent_t e = nullptr;
    if (!ctx->ev_pool.empty()) {
        e = ctx->ev_pool.back();
        ctx->ev_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        return nullptr;
    }
    cudaEventRecord(e, ctx->stream);
    return e;
}

void timer_end(mdg_ctx* ctx, int which, cudaEvent_t start) {
    if (!start) return;
    cudaEvent_t e = nullptr;
    if (!ctx->ev_pool.empty()) {
        e = ctx->ev_pool.back();
        ctx->ev_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        return;
    }
    cudaEventRecord(e, ctx->stream);
    ctx->ev_pending[which].push_back({start, e});
}

int ensure_pinned(mdg_system* sys, size_t bytes) {
    if (bytes <= sys->pin_bytes) return MDG_OK;
    if (sys->host_borrowed) {
        set_error("transfer larger than the owner's pinned staging");
        return MDG_ERR_INVALID;
    }
    if (sys->pin) cudaFreeHost(sys->pin);
    sys->pin = nullptr;
    MDG_CUDA(cudaMallocHost(&sys->pin, bytes));
    sys->pin_bytes = bytes;
    return MDG_OK;
}

int sys_malloc(mdg_system* sys, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    if (sys->pool)
        MDG_CUDA(cudaMallocFromPoolAsync(p, bytes, sys->pool, sys->ctx->stream));
    else
        MDG_CUDA(cudaMalloc(p, bytes));
    sys->dev_bytes += bytes;
    return MDG_OK;
}

void sys_free(mdg_system* sys, void* p, size_t bytes) {
    if (!p) return;
    if (bytes == 0) bytes = 16;
    if (sys->pool)
        cudaFreeAsync(p, sys->ctx->stream);
    else
        cudaFree(p);
    sys->dev_bytes -= std::min(bytes, sys->dev_bytes);
}

// device scratch for host transfers (one per host thread and device; per
// system for pooled systems, whose transfers may overlap other streams)
static int xfer_buffer(mdg_system* sys, size_t bytes, void** out) {
    if (sys->pool) {
        if (bytes > sys->xfer_bytes) {
            sys_free(sys, sys->xfer, sys->xfer_bytes);
            sys->xfer = nullptr;
            sys->xfer_bytes = 0;
            int rc = sys_malloc(sys, &sys->xfer, bytes);
            if (rc) return rc;
            sys->xfer_bytes = bytes;
        }
        *out = sys->xfer;
        return MDG_OK;
    }
    static thread_local void* buf = nullptr;
    static thread_local size_t cap = 0;
    static thread_local int dev = -1;
    if (dev != sys->ctx->device || bytes > cap) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        cap = 0;
        MDG_CUDA(cudaMalloc(&buf, bytes));
        cap = bytes;
        dev = sys->ctx->device;
    }
    *out = buf;
    return MDG_OK;
}

// The per-atom buffers of a system, with their element counts (one table
// for allocation, release and footprint accounting).
template <typename F>
static void for_each_buffer(mdg_system* sys, F&& f) {
    size_t np = std::max<size_t>(sys->np, 32);
    for (int q = 0; q < NF64; ++q)
        for (int b = 0; b < 2; ++b) f((void**)&sys->f64[q][b], np * sizeof(double));
    for (int q = 0; q < 3; ++q)
        for (int b = 0; b < 2; ++b) f((void**)&sys->f32[q][b], np * sizeof(float));
    for (int q = 0; q < NU32; ++q)
        for (int b = 0; b < 2; ++b) f((void**)&sys->u32[q][b], np * sizeof(uint32_t));
    for (int q = 0; q < NU16; ++q)
        for (int b = 0; b < 2; ++b) f((void**)&sys->u16[q][b], np * sizeof(uint16_t));
    for (int a = 0; a < 3; ++a) {
        f((void**)&sys->Rc[a], np * sizeof(double));
        f((void**)&sys->r0[a], np * sizeof(double));
    }
    f((void**)&sys->cellp, np * sizeof(uint32_t));
    f((void**)&sys->pos32, 2 * np * sizeof(int4));
    f((void**)&sys->q0, np * sizeof(int4));
    f((void**)&sys->o0, np * sizeof(float4));
    f((void**)&sys->saved_rcut, np * sizeof(double));
    f((void**)&sys->saved_rns, np * sizeof(double));
    f((void**)&sys->saved_uid, np * sizeof(uint32_t));
    f((void**)&sys->slot_of, np * sizeof(uint32_t));
    f((void**)&sys->bc, np * sizeof(uint8_t));
    f((void**)&sys->Fp64, (size_t)kMaxKinds * np * sizeof(double));
    f((void**)&sys->Fp32, (size_t)kMaxKinds * np * sizeof(float));
    f((void**)&sys->trig32, np * sizeof(float2));
    f((void**)&sys->key, np * sizeof(uint32_t));
    f((void**)&sys->rank, np * sizeof(uint32_t));
    f((void**)&sys->src, np * sizeof(uint32_t));
    f((void**)&sys->ncnt, np * sizeof(uint32_t));
    f((void**)&sys->dstat, sizeof(DevStatus));
    f((void**)&sys->dgrid, sizeof(GridParams));
    f((void**)&sys->red, 16 * sizeof(double));
}

// Device bytes a system of n atoms holds before its first list (the bin,
// list and transfer buffers come on top).
size_t system_base_bytes(size_t n) {
    mdg_system probe;
    probe.np = (n + 31) & ~size_t(31);
    size_t total = 0;
    for_each_buffer(&probe, [&](void**, size_t b) { total += b; });
    return total;
}

int system_alloc(mdg_system* sys) {
    int rc = MDG_OK;
    for_each_buffer(sys, [&](void** p, size_t b) {
        if (rc == MDG_OK) rc = sys_malloc(sys, p, b);
    });
    if (rc) return rc;
    if (!sys->host_borrowed) {
        MDG_CUDA(cudaMallocHost((void**)&sys->hgrid, sizeof(GridParams)));
        MDG_CUDA(cudaMallocHost((void**)&sys->hstat, sizeof(DevStatus)));
        MDG_CUDA(cudaMallocHost((void**)&sys->hred, 16 * sizeof(double)));
    }
    size_t np = std::max<size_t>(sys->np, 32);
    cudaStream_t st = sys->ctx->stream;
    if (sys->lazy_init) return MDG_OK;
    MDG_CUDA(cudaMemsetAsync(sys->dstat, 0, sizeof(DevStatus), st));
    MDG_CUDA(cudaMemsetAsync(sys->ncnt, 0, np * sizeof(uint32_t), st));
    MDG_CUDA(cudaMemsetAsync(sys->bc, 0, np, st));
    MDG_CUDA(cudaMemsetAsync(sys->Fp64, 0, (size_t)kMaxKinds * np * sizeof(double), st));
    MDG_CUDA(cudaMemsetAsync(sys->trig32, 0, np * sizeof(float2), st));
    for (int a = 0; a < 3; ++a) MDG_CUDA(cudaMemsetAsync(sys->Rc[a], 0, np * sizeof(double), st));
    if (sys->n) {
        k_iota<<<nblk(sys->n), kBlock, 0, st>>>((int)sys->n, sys->u32[ORIG][0], sys->slot_of);
        MDG_LAUNCHED(sys->ctx);
    }
    // a pooled system's buffers are stream-ordered: nothing to wait for
    if (!sys->pool) MDG_CUDA(cudaStreamSynchronize(st));
    return MDG_OK;
}

void system_free(mdg_system* sys) {
    if (sys->run_exec) cudaGraphExecDestroy(sys->run_exec);
    if (sys->run_graph) cudaGraphDestroy(sys->run_graph);
    sys->run_exec = nullptr;
    sys->run_graph = nullptr;
    sys_free(sys, sys->dcounter, sizeof(unsigned long long));
    for_each_buffer(sys, [&](void** p, size_t b) {
        sys_free(sys, *p, b);
        *p = nullptr;
    });
    sys_free(sys, sys->bin_count, sys->bin_cap * sizeof(uint32_t));
    sys_free(sys, sys->bin_start, sys->bin_cap * sizeof(uint32_t));
    sys_free(sys, sys->scan_tmp, sys->scan_cap * sizeof(uint32_t));
    sys_free(sys, sys->part, sys->part_cap * 8 * sizeof(double));
    sys_free(sys, sys->nbr, (size_t)sys->K * sys->np * sizeof(uint32_t));
    sys_free(sys, sys->cutbits, (size_t)sys->cut_words * sys->np * sizeof(uint32_t));
    sys->cutbits = nullptr;
    sys->cut_words = 0;
    sys_free(sys, sys->xfer, sys->xfer_bytes);
    sys_free(sys, sys->step_io, sys->step_io_bytes);
    sys->step_io = nullptr;
    sys->step_io_bytes = 0;
    for (cudaEvent_t& e : sys->step_ev) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
    }
    if (!sys->host_borrowed) {
        if (sys->hcounter) cudaFreeHost(sys->hcounter);
        cudaFreeHost(sys->hgrid);
        cudaFreeHost(sys->hstat);
        cudaFreeHost(sys->hred);
        if (sys->pin) cudaFreeHost(sys->pin);
    }
}

// ---------------------------------------------------------------------------
// potentials: tables, spline slopes (EAM::init_spline, EAM.cxx:603-686)
// ---------------------------------------------------------------------------
static void init_spline(const double* y, double* z, double H1, size_t N, int ib) {
    std::vector<double> a(N, 2.0), b(N, 0.0), c(N, 0.0), d(N, 0.0);
    std::vector<double> s(N + 1, 0.0), t(N + 1, 0.0), u(N + 1, 0.0), v(N + 1, 0.0), w(N + 1, 0.0);
    b[0] = 1.0;
    c[0] = 0.0;
    d[0] = 3.0 * H1 * (y[1] - y[0]);
    b[N - 1] = 0.0;
    if (ib == 1) {
        c[N - 1] = 0.0;
        d[N - 1] = 0.0;
    } else if (ib == 2) {
        c[N - 1] = 1.0;
        d[N - 1] = 3.0 * H1 * (y[N - 1] - y[N - 2]);
    }
    for (size_t i = 1; i < N - 1; i++) {
        c[i] = 0.5;
        b[i] = 0.5;
        d[i] = 1.5 * H1 * (y[i + 1] - y[i - 1]);
    }
    u[0] = 0.0;
    v[0] = 0.0;
    w[0] = 1.0;
    for (size_t i = 0; i < N; i++) {
        double rp = -1.0 / (a[i] + c[i] * v[i]);
        v[i + 1] = rp * b[i];
        u[i + 1] = rp * (c[i] * u[i] - d[i]);
        w[i + 1] = rp * c[i] * w[i];
    }
    s[N - 1] = 1.0;
    t[N - 1] = 0.0;
    for (long i = (long)N - 2; i >= 0; i--) {
        s[i] = v[i + 1] * s[i + 1] + w[i + 1];
        t[i] = v[i + 1] * t[i + 1] + u[i + 1];
    }
    for (size_t i = 0; i < N; ++i) z[i] = 0.0;
    z[N - 1] = (d[N - 1] - b[N - 1] * t[0] - c[N - 1] * t[N - 2]) /
               (a[N - 1] + b[N - 1] * s[0] + c[N - 1] * s[N - 2]);
    // The reference reads z[i] (zero on entry) in this update.
    for (size_t i = 0; i < N - 1; i++) z[i] = s[i] * z[i] + t[i];
}

// Cubic coefficients of the Hermite piece on [x_n, x_n + h] in u = (x - x_n)/h:
// value = y_n + u*(h z_n) + u^2*(-h b) + u^3*(h a) with the reference's a, b.
static void cubic_coeffs(const std::vector<double>& y, const std::vector<double>& z, double h, int N,
                         std::vector<float4>& out) {
    out.resize(N);
    double h1 = 1.0 / h;
    for (int n = 0; n < N; ++n) {
        double m = (y[n + 1] - y[n]) * h1;
        double aa = (z[n + 1] - m) - (m - z[n]);
        double bb = aa - (m - z[n]);
        out[n] = make_float4((float)y[n], (float)(h * z[n]), (float)(-h * bb), (float)(h * aa));
    }
}

// Per-interval polynomials of the force pass, in u on [x_n, x_n + h] with
// x_n = n h, from the FP64 pieces of the rho and r*phi (Vpar) splines:
//   W(u)  = V'(r) r - V(r)  (cubic: the V piece's derivative times r = (n + u) h,
//           minus the piece itself), row .x..w = W0..W3;
//   D(u)  = rho'(r)         (quadratic: the rho piece's derivative), row .x..z;
// so that the EAM pair force over r is ((F'_i + F'_j) D + W / r^2) / r
// (EAM.cxx:417-463) with every coefficient rounded once from FP64.
static void force_rows(const std::vector<double>& ry, const std::vector<double>& rz, const std::vector<double>& vy,
                       const std::vector<double>& vz, double h, int N, std::vector<float4>& out) {
    out.resize(2 * (size_t)N);
    const double h1 = 1.0 / h;
    for (int n = 0; n < N; ++n) {
        // V piece: v0 + v1 u + v2 u^2 + v3 u^3 (the reference's a, b form)
        double m = (vy[n + 1] - vy[n]) * h1;
        double aa = (vz[n + 1] - m) - (m - vz[n]);
        double bb = aa - (m - vz[n]);
        const double v0 = vy[n], v1 = h * vz[n], v2 = -h * bb, v3 = h * aa;
        const double k = (double)n;
        out[2 * (size_t)n] = make_float4((float)(v1 * k - v0), (float)(2.0 * v2 * k), (float)(v2 + 3.0 * v3 * k),
                                         (float)(2.0 * v3));
        // rho piece's derivative in r: (c1 + 2 c2 u + 3 c3 u^2) / h
        m = (ry[n + 1] - ry[n]) * h1;
        aa = (rz[n + 1] - m) - (m - rz[n]);
        bb = aa - (m - rz[n]);
        out[2 * (size_t)n + 1] = make_float4((float)rz[n], (float)(-2.0 * bb), (float)(3.0 * aa), 0.f);
    }
}

int pot_upload(mdg_potential* p, int device) {
    if ((p->type != POT_EAM && p->type != POT_TAB) || p->device == device) return MDG_OK;
    if (p->d_tab64) cudaFree(p->d_tab64);
    if (p->d_tab32) cudaFree(p->d_tab32);
    p->d_tab64 = nullptr;
    p->d_tab32 = nullptr;
    size_t nr = (size_t)p->Nr1 + 1, nh = (size_t)p->Nrh1 + 1;
    std::vector<double> h64;
    h64.reserve(4 * nr + 2 * nh);
    for (auto* v : {&p->Rho, &p->dRho, &p->Vpar, &p->dVpar}) h64.insert(h64.end(), v->begin(), v->end());
    for (auto* v : {&p->Femb, &p->dFemb}) h64.insert(h64.end(), v->begin(), v->end());
    std::vector<float4> rc, vc, fc, h32;
    cubic_coeffs(p->Rho, p->dRho, p->dr, p->Nr1, rc);
    cubic_coeffs(p->Vpar, p->dVpar, p->dr, p->Nr1, vc);
    cubic_coeffs(p->Femb, p->dFemb, p->drh, p->Nrh1, fc);
    h32.insert(h32.end(), rc.begin(), rc.end());
    h32.insert(h32.end(), vc.begin(), vc.end());
    h32.insert(h32.end(), fc.begin(), fc.end());
    // the force pass's W and D rows of each interval (32 bytes), read with
    // one load, 32-byte aligned
    if (h32.size() & 1) h32.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    std::vector<float4> fr;
    force_rows(p->Rho, p->dRho, p->Vpar, p->dVpar, p->dr, p->Nr1, fr);
    h32.insert(h32.end(), fr.begin(), fr.end());
    MDG_CUDA(cudaSetDevice(device));
    MDG_CUDA(cudaMalloc(&p->d_tab64, h64.size() * sizeof(double)));
    MDG_CUDA(cudaMalloc(&p->d_tab32, h32.size() * sizeof(float4)));
    MDG_CUDA(cudaMemcpy(p->d_tab64, h64.data(), h64.size() * sizeof(double), cudaMemcpyHostToDevice));
    MDG_CUDA(cudaMemcpy(p->d_tab32, h32.data(), h32.size() * sizeof(float4), cudaMemcpyHostToDevice));
    p->device = device;
    return MDG_OK;
}

// Table-less slots (no potential, LJsCut) point every table at `z64` /
// `z32`, kZeroRows rows of zeros, so that no kernel load sees a null pointer.
static void zero_tables(PotParams& P, const double* z64, const float4* z32) {
    P.Rho = P.dRho = P.Vpar = P.dVpar = P.Femb = P.dFemb = z64;
    P.rho_c = P.v_c = P.f_c = P.rv_c = z32;
}

static void fill_params(const mdg_potential* p, PotParams& P, const double* z64, const float4* z32) {
    memset(&P, 0, sizeof(P));
    zero_tables(P, z64, z32);
    if (!p) return;
    P.type = p->type;
    P.R2cut = p->rcut * p->rcut;
    P.r2cut_f = (float)P.R2cut;
    if (p->type == 1) {
        P.a = p->a;
        P.s6 = p->s6;
        P.lj1 = p->lj1;
        P.lj2 = p->lj2;
        P.factor = p->factor;
        P.lj1_f = (float)p->lj1;
        P.lj2_f = (float)p->lj2;
        P.mhf_f = (float)(-0.5 * p->factor);
    } else if (p->type == POT_LJS) {
        P.ljs_rVr1 = p->ljs_rVr1;
        P.ljs_rVr2 = p->ljs_rVr2;
        P.ljs_aLJ = p->ljs_aLJ;
        P.ljs_bLJ = p->ljs_bLJ;
        P.ljs_aLJ3 = p->ljs_aLJ3;
        P.ljs_bLJ2 = p->ljs_bLJ2;
        P.ljs_aVr = p->ljs_aVr;
        P.ljs_aVr2 = p->ljs_aVr2;
        P.ljs_rVr1_f = (float)p->ljs_rVr1;
        P.ljs_rVr2_f = (float)p->ljs_rVr2;
        P.ljs_aLJ_f = (float)p->ljs_aLJ;
        P.ljs_bLJ_f = (float)p->ljs_bLJ;
        P.ljs_aVr2_f = (float)p->ljs_aVr2;
    } else if (p->type == POT_EAM || p->type == POT_TAB) {
        size_t nr = (size_t)p->Nr1 + 1, nh = (size_t)p->Nrh1 + 1;
        P.Nr1 = p->Nr1;
        P.Nrh1 = p->Nrh1;
        P.dr = p->dr;
        P.drh = p->drh;
        P.dr1 = p->dr1;
        P.drh1 = p->drh1;
        P.Rho = p->d_tab64;
        P.dRho = p->d_tab64 + nr;
        P.Vpar = p->d_tab64 + 2 * nr;
        P.dVpar = p->d_tab64 + 3 * nr;
        P.Femb = p->d_tab64 + 4 * nr;
        P.dFemb = p->d_tab64 + 4 * nr + nh;
        P.rho_c = p->d_tab32;
        P.v_c = p->d_tab32 + p->Nr1;
        P.f_c = p->d_tab32 + 2 * p->Nr1;
        P.rv_c = p->d_tab32 + ((2 * (size_t)p->Nr1 + p->Nrh1 + 1) & ~size_t(1));
        P.inv_dr_f = (float)(1.0 / p->dr);
        P.inv_drh_f = (float)(1.0 / p->drh);
        P.dr1_f = (float)p->dr1;
        P.drh_f = (float)p->drh;
    }
}

}  // namespace mdg

using namespace mdg;

// solver + system binding: the PotSet, the thermostat's terms and the zero
// table live in one device block per (solver, device); the PotSet is
// rebuilt when potentials change, the terms whenever they differ from the
// last copy (before any capture, so a graph reads the current values).
struct SolverBlob {
    PotSet ps;
    ThermoDev th;
    alignas(32) float4 z32[2 * kZeroRows];
    double z64[2 * kZeroRows];
};

struct SolverDev {
    PotSet host;
    PotSet* dev = nullptr;  // start of the SolverBlob
    int device = -1;
    int version = -1;
    ThermoDev th_host{};
    int th_valid = 0;
};

struct mdg_solver_ext {
    mdg_solver s;
    SolverDev d;
    int version = 0;
};

static SolverBlob* blob_of(SolverDev& d) { return reinterpret_cast<SolverBlob*>(d.dev); }

static mdg_solver_ext* ext(mdg_solver* s) { return reinterpret_cast<mdg_solver_ext*>(s); }

namespace mdg {
int potset_build(mdg_solver* s, mdg_system* sys, PotSet* out) {
    mdg_solver_ext* e = ext(s);
    int dev = sys->ctx->device;
    if (e->d.device == dev && e->d.version == e->version && e->d.dev) {
        e->d.host.periodic = s->periodic;
        if (out) *out = e->d.host;
        return MDG_OK;
    }
    if (!e->d.dev || e->d.device != dev) {
        if (e->d.dev) cudaFree(e->d.dev);
        e->d.dev = nullptr;
        e->d.th_valid = 0;
        MDG_CUDA(cudaMalloc(&e->d.dev, sizeof(SolverBlob)));
        MDG_CUDA(cudaMemset(e->d.dev, 0, sizeof(SolverBlob)));
    }
    SolverBlob* b = blob_of(e->d);
    PotSet ps;
    memset(&ps, 0, sizeof(ps));
    ps.nkinds = s->multi ? s->nkinds : 1;
    ps.multi = s->multi;
    ps.periodic = s->periodic;
    for (int i = 0; i < kMaxKinds; ++i)
        for (int j = 0; j < kMaxKinds; ++j) {
            mdg_potential* p = i < ps.nkinds && j < ps.nkinds ? s->pot[i][j] : nullptr;
            if (p) {
                int rc = pot_upload(p, dev);
                if (rc) return rc;
                if (p->type == POT_EAM) ps.any_eam = 1;
                if (p->type == POT_LJCUT) ps.any_lj = 1;
                if (p->type == POT_LJS) ps.any_ljs = 1;
                if (p->type == POT_TAB) ps.any_tab = 1;
            }
            fill_params(p, ps.p[i][j], b->z64, b->z32);
        }
    MDG_CUDA(cudaMemcpy(e->d.dev, &ps, sizeof(PotSet), cudaMemcpyHostToDevice));
    e->d.host = ps;
    e->d.device = dev;
    e->d.version = e->version;
    if (out) *out = ps;
    return MDG_OK;
}
}  // namespace mdg

namespace mdg {
// Device terms of the solver's thermostat (null without one); refreshed in
// check_ready, read by the launches.
const ThermoDev* thermo_of(mdg_solver* s) {
    if (!s->thermo) return nullptr;
    return &blob_of(ext(s)->d)->th;
}
}  // namespace mdg

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

const char* mdg_last_error(void) { return g_err.c_str(); }
const char* mdg_version(void) { return "mdg 0.1 (sm_103a)"; }

int mdg_ctx_create(int device, mdg_ctx** out) {
    if (!out) return MDG_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error("no CUDA device available (libmdg has no CPU fallback)");
        return MDG_ERR_NODEV;
    }
    if (device < 0 || device >= count) {
        set_error("device index out of range");
        return MDG_ERR_INVALID;
    }
    MDG_CUDA(cudaSetDevice(device));
    mdg_ctx* c = new mdg_ctx();
    c->device = device;
    cudaError_t e2 = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e2 != cudaSuccess) {
        delete c;
        return cuda_status(e2, "cudaStreamCreate");
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    *out = c;
    return MDG_OK;
}

static void ctx_release(mdg_ctx* ctx) {
    if (--ctx->refs > 0) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (int w = 0; w < 5; ++w)
        for (auto& pr : ctx->ev_pending[w]) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    if (ctx->io_stream) cudaStreamDestroy(ctx->io_stream);
    delete ctx;
}

int mdg_ctx_destroy(mdg_ctx* ctx) {
    if (!ctx || ctx->closed) return MDG_ERR_INVALID;
    ctx->closed = 1;
    ctx_release(ctx);
    return MDG_OK;
}

int mdg_ctx_synchronize(mdg_ctx* ctx) {
    if (!ctx) return MDG_ERR_INVALID;
    MDG_CUDA(cudaStreamSynchronize(ctx->stream));
    return MDG_OK;
}

int mdg_ctx_stream(mdg_ctx* ctx, void** stream) {
    if (!ctx || !stream) return MDG_ERR_INVALID;
    *stream = (void*)ctx->stream;
    return MDG_OK;
}

int mdg_ctx_launch_count(mdg_ctx* ctx, uint64_t* out) {
    if (!ctx || !out) return MDG_ERR_INVALID;
    *out = ctx->launches;
    return MDG_OK;
}

int mdg_ctx_set_timing(mdg_ctx* ctx, int on) {
    if (!ctx) return MDG_ERR_INVALID;
    MDG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->timing = on ? 1 : 0;
    for (int w = 0; w < 5; ++w) {
        for (auto& pr : ctx->ev_pending[w]) {
            ctx->ev_pool.push_back(pr.first);
            ctx->ev_pool.push_back(pr.second);
        }
        ctx->ev_pending[w].clear();
        ctx->stage_ms[w] = 0.0;
        ctx->stage_n[w] = 0;
    }
    return MDG_OK;
}

int mdg_ctx_stage_time(mdg_ctx* ctx, int which, double* total_ms, uint64_t* launches) {
    if (!ctx || which < 0 || which > 4 || !total_ms) return MDG_ERR_INVALID;
    MDG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int w = 0; w < 5; ++w) {
        for (auto& pr : ctx->ev_pending[w]) {
            float ms = 0.f;
            MDG_CUDA(cudaEventElapsedTime(&ms, pr.first, pr.second));
            ctx->stage_ms[w] += ms;
            ctx->stage_n[w]++;
            ctx->ev_pool.push_back(pr.first);
            ctx->ev_pool.push_back(pr.second);
        }
        ctx->ev_pending[w].clear();
    }
    *total_ms = ctx->stage_ms[which];
    if (launches) *launches = ctx->stage_n[which];
    return MDG_OK;
}

}  // extern "C"

namespace mdg {

int system_create(mdg_ctx* ctx, const mdg_domain* domain, size_t n, const SystemMemory* mem, mdg_system** out) {
    *out = nullptr;
    if (n >= kMaxAtoms) {
        set_error("system too large: at most 2^25 - 1 atoms per system");
        return MDG_ERR_INVALID;
    }
    MDG_CUDA(cudaSetDevice(ctx->device));
    mdg_system* s = new mdg_system();
    s->ctx = ctx;
    s->dom = *domain;
    double zs = domain->bmax[2] - domain->bmin[2], ys = domain->bmax[1] - domain->bmin[1];
    s->dim = std::fabs(-zs) > 1e-15 ? 3 : std::fabs(-ys) > 1e-15 ? 2 : 1;
    s->n = n;
    s->np = (n + 31) & ~size_t(31);
    if (mem) {
        s->lazy_init = mem->lazy_init;
        s->pool = mem->pool;
        s->host_borrowed = 1;
        s->hgrid = mem->hgrid;
        s->hstat = mem->hstat;
        s->hred = mem->hred;
        s->hcounter = mem->hcounter;
        s->pin = mem->pin;
        s->pin_bytes = mem->pin_bytes;
    }
    int rc = system_alloc(s);
    if (rc) {
        system_free(s);
        delete s;
        return rc;
    }
    ctx->refs++;
    *out = s;
    return MDG_OK;
}

// Frees a system without waiting: pooled buffers are released in stream
// order behind its last work.
void system_release(mdg_system* sys) {
    mdg_ctx* ctx = sys->ctx;
    cudaSetDevice(ctx->device);
    if (!sys->pool) cudaStreamSynchronize(ctx->stream);
    system_free(sys);
    delete sys;
    ctx_release(ctx);
}

}  // namespace mdg

extern "C" {

int mdg_system_create(mdg_ctx* ctx, const mdg_domain* domain, size_t n, mdg_system** out) {
    if (!ctx || !domain || !out) return MDG_ERR_INVALID;
    return system_create(ctx, domain, n, nullptr, out);
}

int mdg_system_destroy(mdg_system* sys) {
    if (!sys) return MDG_ERR_INVALID;
    system_release(sys);
    return MDG_OK;
}

int mdg_system_size(mdg_system* sys, size_t* n) {
    if (!sys || !n) return MDG_ERR_INVALID;
    *n = sys->n;
    return MDG_OK;
}

static int sync_forces64(mdg_system* sys);

}  // extern "C"

namespace mdg {

// Stages the atoms through the system's pinned buffer and scatters them on
// the device; does not wait (the pinned buffer is busy until the stream has
// passed this point).
int upload_atoms_enqueue(mdg_system* sys, const mdg_atom* atoms, size_t n) {
    cudaStream_t st = sys->ctx->stream;
    size_t bytes = n * sizeof(mdg_atom);
    void* dbuf;
    int rc = ensure_pinned(sys, bytes);
    if (rc) return rc;
    rc = xfer_buffer(sys, bytes, &dbuf);
    if (rc) return rc;
    memcpy(sys->pin, atoms, bytes);
    MDG_CUDA(cudaMemcpyAsync(dbuf, sys->pin, bytes, cudaMemcpyHostToDevice, st));
    k_atoms_in<<<nblk(n), kBlock, 0, st>>>(xfer_args(sys), (const mdg_atom*)dbuf);
    MDG_LAUNCHED(sys->ctx);
    sys->force_prec = MDG_PREC_FP64;
    sys->fp_ok = 0;  // nc replaced
    if (sys->have_list) {
        rc = launch_offsets(sys);
        if (rc) return rc;
    }
    return MDG_OK;
}

// Gathers the atoms (caller order, FP64 forces) into the system's pinned
// buffer; does not wait.
int download_atoms_enqueue(mdg_system* sys, size_t n) {
    cudaStream_t st = sys->ctx->stream;
    size_t bytes = n * sizeof(mdg_atom);
    void* dbuf;
    int rc = ensure_pinned(sys, bytes);
    if (rc) return rc;
    rc = xfer_buffer(sys, bytes, &dbuf);
    if (rc) return rc;
    rc = sync_forces64(sys);
    if (rc) return rc;
    rc = settle_outputs(sys);
    if (rc) return rc;
    k_atoms_out<<<nblk(n), kBlock, 0, st>>>(xfer_args(sys), sys->bc, (mdg_atom*)dbuf);
    MDG_LAUNCHED(sys->ctx);
    MDG_CUDA(cudaMemcpyAsync(sys->pin, dbuf, bytes, cudaMemcpyDeviceToHost, st));
    return MDG_OK;
}

}  // namespace mdg

extern "C" {

int mdg_system_upload_atoms(mdg_system* sys, const mdg_atom* atoms, size_t n) {
    if (!sys || (!atoms && n) || n != sys->n) {
        set_error("atom count differs from the system size");
        return MDG_ERR_INVALID;
    }
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    int rc = upload_atoms_enqueue(sys, atoms, n);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

static int sync_forces64(mdg_system* sys) {
    if (sys->force_prec == MDG_PREC_MIXED) {
        int rc = launch_force_copy(sys, 1);
        if (rc) return rc;
        sys->force_prec = MDG_PREC_FP64;
    }
    return MDG_OK;
}

int mdg_system_download_atoms(mdg_system* sys, mdg_atom* atoms, size_t n) {
    if (!sys || (!atoms && n) || n != sys->n) return MDG_ERR_INVALID;
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    int rc = download_atoms_enqueue(sys, n);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    memcpy(atoms, sys->pin, n * sizeof(mdg_atom));
    return MDG_OK;
}

// Enqueues one xyz transfer (caller order <-> slot order through the
// transfer buffer); `sync` waits for it (the host buffer is then free).
static int vec_io(mdg_system* sys, double* host, int field, int in, int sync = 1) {
    if (!sys || !host) return MDG_ERR_INVALID;
    size_t n = sys->n;
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    cudaStream_t st = sys->ctx->stream;
    size_t bytes = n * 3 * sizeof(double);
    void* dbuf;
    int rc = xfer_buffer(sys, bytes, &dbuf);
    if (rc) return rc;
    int c = sys->cur;
    if (in) {
        MDG_CUDA(cudaMemcpyAsync(dbuf, host, bytes, cudaMemcpyHostToDevice, st));
        k_vec_in<<<nblk(n), kBlock, 0, st>>>((int)n, sys->slot_of, (const double*)dbuf, sys->f64[field][c],
                                             sys->f64[field + 1][c], sys->f64[field + 2][c]);
        MDG_LAUNCHED(sys->ctx);
        if (field == RX && sys->have_list) {
            rc = launch_offsets(sys);
            if (rc) return rc;
        }
        if (sync) MDG_CUDA(cudaStreamSynchronize(st));
    } else {
        if (field == FX) {
            rc = sync_forces64(sys);
            if (rc) return rc;
        }
        k_vec_out<<<nblk(n), kBlock, 0, st>>>((int)n, sys->slot_of, sys->f64[field][c], sys->f64[field + 1][c],
                                              sys->f64[field + 2][c], (double*)dbuf);
        MDG_LAUNCHED(sys->ctx);
        MDG_CUDA(cudaMemcpyAsync(host, dbuf, bytes, cudaMemcpyDeviceToHost, st));
        if (sync) MDG_CUDA(cudaStreamSynchronize(st));
    }
    return MDG_OK;
}

int mdg_system_set_positions(mdg_system* sys, const double* xyz) { return vec_io(sys, (double*)xyz, RX, 1); }
int mdg_system_get_positions(mdg_system* sys, double* xyz) { return vec_io(sys, xyz, RX, 0); }
int mdg_system_set_velocities(mdg_system* sys, const double* xyz) { return vec_io(sys, (double*)xyz, VX, 1); }
int mdg_system_get_velocities(mdg_system* sys, double* xyz) { return vec_io(sys, xyz, VX, 0); }
int mdg_system_get_forces(mdg_system* sys, double* xyz) { return vec_io(sys, xyz, FX, 0); }

// ---- Verlet list -----------------------------------------------------------
int mdg_nlist_update(mdg_system* sys, double kbuf, int half) {
    if (!sys) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    int rc = nlist_build(sys, kbuf, half ? 1 : 0);  // it also refreshes the rebuild thresholds
    if (rc && rc != MDG_ERR_RANGE) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return rc;
}

int mdg_nlist_decide(mdg_system* sys, int* need) {
    if (!sys || !need) return MDG_ERR_INVALID;
    if (!sys->have_list) {
        *need = 1;
        return MDG_OK;
    }
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    cudaStream_t st = sys->ctx->stream;
    MDG_CUDA(cudaMemsetAsync(&sys->dstat->need_rebuild, 0, sizeof(uint32_t), st));
    int rc = launch_decide(sys);
    if (rc) return rc;
    MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    *need = sys->hstat->need_rebuild ? 1 : 0;
    return MDG_OK;
}

int mdg_nlist_total(mdg_system* sys, size_t* total) {
    if (!sys || !total) return MDG_ERR_INVALID;
    if (!sys->have_list) return MDG_ERR_STATE;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    std::vector<uint64_t> off;
    int rc = nlist_export_offsets(sys, off);
    if (rc) return rc;
    *total = (size_t)off[sys->n];
    return MDG_OK;
}

int mdg_nlist_export(mdg_system* sys, uint64_t* offsets, uint64_t* idx, size_t cap) {
    if (!sys || !offsets) return MDG_ERR_INVALID;
    if (!sys->have_list) return MDG_ERR_STATE;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    std::vector<uint64_t> off;
    int rc = nlist_export_offsets(sys, off);
    if (rc) return rc;
    const size_t total = (size_t)off[sys->n];
    if (total > cap || (!idx && total)) {
        set_error("export capacity too small");
        return MDG_ERR_INVALID;
    }
    rc = nlist_export_entries(sys, off, idx);
    if (rc) return rc;
    memcpy(offsets, off.data(), off.size() * sizeof(uint64_t));
    return MDG_OK;
}

int mdg_nlist_grid(mdg_system* sys, int32_t ints[9], double dbls[3]) {
    if (!sys || !ints || !dbls) return MDG_ERR_INVALID;
    if (!sys->have_list) return MDG_ERR_STATE;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    // the grid of the last rebuild, which may have run inside a device loop
    GridParams g;
    MDG_CUDA(cudaMemcpyAsync(&g, sys->dgrid, sizeof(GridParams), cudaMemcpyDeviceToHost, sys->ctx->stream));
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    for (int a = 0; a < 3; ++a) {
        ints[a] = g.dom_n[a];
        ints[3 + a] = g.offset[a];
        ints[6 + a] = g.num[a];
        dbls[a] = g.cs[a];
    }
    return MDG_OK;
}

int mdg_nlist_rebuilds(mdg_system* sys, uint64_t* count) {
    if (!sys || !count) return MDG_ERR_INVALID;
    *count = sys->rebuilds;
    return MDG_OK;
}

// VerletList::list_for (verlet-list.cxx:251-276), evaluated on the host from
// the device's last grid and positions; radius = Grid::cell_size().
int mdg_nlist_list_for(mdg_system* sys, const double x[3], uint64_t* out, size_t cap, size_t* count) {
    if (!sys || !x || !count || (!out && cap)) return MDG_ERR_INVALID;
    if (!sys->have_list) return MDG_ERR_STATE;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    std::vector<uint64_t> found;
    int rc = nlist_list_for(sys, x, found);
    if (rc) return rc;
    *count = found.size();
    for (size_t k = 0; k < found.size() && k < cap; ++k) out[k] = found[k];
    return MDG_OK;
}

int mdg_nlist_sort(mdg_system* sys, mdg_atom* atoms, size_t n, mdg_atom* sorted) {
    if (!sys || ((!atoms || !sorted) && n) || (n && atoms == sorted)) return MDG_ERR_INVALID;
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    // the atoms go through a scratch system on the same device and domain:
    // its rebuild wraps them and bins them on the grid built from them
    mdg_system* tmp = nullptr;
    int rc = mdg_system_create(sys->ctx, &sys->dom, n, &tmp);
    if (rc) return rc;
    std::vector<uint32_t> perm(n);
    std::vector<double> r(3 * n);
    uint32_t* dperm = nullptr;
    rc = mdg_system_upload_atoms(tmp, atoms, n);
    int range = 0;
    if (!rc) {
        rc = nlist_build(tmp, -1.0, 0);
        if (rc == MDG_ERR_RANGE) {  // clamped into the nearest cell, as update() does
            range = 1;
            rc = MDG_OK;
        }
    }
    if (!rc && cudaMalloc(&dperm, n * sizeof(uint32_t)) != cudaSuccess) rc = MDG_ERR_NOMEM;
    if (!rc) rc = nlist_sort_perm(tmp, dperm);
    if (!rc && cudaMemcpy(perm.data(), dperm, n * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = MDG_ERR_CUDA;
    if (!rc) rc = mdg_system_get_positions(tmp, r.data());
    if (dperm) cudaFree(dperm);
    mdg_system_destroy(tmp);
    if (rc) return rc;
    // the caller's atoms take the wrapped positions (put_atoms_in_cells,
    // verlet-list.cxx:182-185); the copy is every record as it is, reordered
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) atoms[i].r[a] = r[3 * i + a];
    for (size_t p = 0; p < n; ++p) sorted[p] = atoms[perm[p]];
    if (range) {
        set_error("an atom lies outside the cell grid; it was sorted into the nearest cell");
        return MDG_ERR_RANGE;
    }
    return MDG_OK;
}

// ---- potentials ----------------------------------------------------------
int mdg_pot_ljcut_create(double a, double s, double rcut, mdg_potential** out) {
    if (!out || !(rcut > 0.0)) return MDG_ERR_INVALID;
    mdg_potential* p = new mdg_potential();
    p->type = 1;
    p->rcut = rcut;
    p->a = a;
    p->s = s;
    p->s6 = std::pow(s, 6);
    p->lj1 = 2 * p->s6;
    p->lj2 = 1.;
    p->factor = 48. * p->a * p->s6;
    *out = p;
    return MDG_OK;
}

int mdg_pot_eam_create(double rcut, const double* Femb, const double* Rho, const double* Vpar, int Nr1, double dr,
                       int Nrh1, double drh, mdg_potential** out) {
    if (!out || !Femb || !Rho || !Vpar || Nr1 < 3 || Nrh1 < 3 || !(dr > 0) || !(drh > 0)) {
        set_error("invalid EAM tables");
        return MDG_ERR_INVALID;
    }
    mdg_potential* p = new mdg_potential();
    p->type = 2;
    p->rcut = rcut;
    p->Nr1 = Nr1;
    p->Nrh1 = Nrh1;
    p->dr = dr;
    p->drh = drh;
    p->dr1 = 1.0 / dr;
    p->drh1 = 1.0 / drh;
    p->Rho.assign(Rho, Rho + Nr1);
    p->Vpar.assign(Vpar, Vpar + Nr1);
    p->Femb.assign(Femb, Femb + Nrh1);
    p->dRho.assign(Nr1 + 1, 0.0);
    p->dVpar.assign(Nr1 + 1, 0.0);
    p->dFemb.assign(Nrh1 + 1, 0.0);
    init_spline(p->Vpar.data(), p->dVpar.data(), p->dr1, Nr1, 1);
    init_spline(p->Rho.data(), p->dRho.data(), p->dr1, Nr1, 1);
    init_spline(p->Femb.data(), p->dFemb.data(), p->drh1, Nrh1, 2);
    // one padding element: the reference reads index N at the table edge
    p->Rho.push_back(p->Rho.back());
    p->Vpar.push_back(p->Vpar.back());
    p->Femb.push_back(p->Femb.back());
    p->dRho[Nr1] = p->dRho[Nr1 - 1];
    p->dVpar[Nr1] = p->dVpar[Nr1 - 1];
    p->dFemb[Nrh1] = p->dFemb[Nrh1 - 1];
    *out = p;
    return MDG_OK;
}

int mdg_pot_eam_create_from_file(const char* path, mdg_potential** out) {
    // EAM::EAM(std::string) (EAM.cxx:55-87)
    if (!path || !out) return MDG_ERR_INVALID;
    std::ifstream file(path);
    if (!file.is_open()) {
        set_error(std::string("cannot open EAM file: ") + path);
        return MDG_ERR_IO;
    }
    const double N_a = 6.02214076e+23, Qelectron = 1.602176634e-19;
    const double UnMass = 1e-3 / N_a, UnLeng = 1e-9, UnTime = 1e-12;
    const double UnEnrg = UnMass * (UnLeng / UnTime) * (UnLeng / UnTime);
    std::string line;
    for (int k = 0; k < 4; ++k) std::getline(file, line);
    int Nrh1 = 0, Nr1 = 0, Z = 0;
    double drh = 0, dr = 0, rcut = 0, M = 0, Ecoh = 0;
    std::string lattice;
    file >> Nrh1 >> drh >> Nr1 >> dr >> rcut;
    file >> Z >> M >> Ecoh >> lattice;
    if (!file || Nrh1 < 3 || Nr1 < 3) {
        set_error("malformed EAM setfl header");
        return MDG_ERR_IO;
    }
    dr /= 10;
    rcut /= 10;
    std::vector<double> F(Nrh1), R(Nr1), V(Nr1);
    for (int i = 0; i < Nrh1; ++i) {
        file >> F[i];
        F[i] *= Qelectron / UnEnrg;
    }
    for (int i = 0; i < Nr1; ++i) file >> R[i];
    for (int i = 0; i < Nr1; ++i) {
        file >> V[i];
        V[i] *= Qelectron / (10 * UnEnrg);
    }
    if (!file) {
        set_error("EAM file ended before all tables were read");
        return MDG_ERR_IO;
    }
    return mdg_pot_eam_create(rcut, F.data(), R.data(), V.data(), Nr1, dr, Nrh1, drh, out);
}

int mdg_pot_ljs_create(double aVr, double rVr, double rcut, mdg_potential** out) {
    // LJs::LJs (LJs.cxx:7-29), same operation order
    if (!out || !(rcut > 0.0) || !(rVr > 0.0)) return MDG_ERR_INVALID;
    const double X2min = 1.2599210498948732;
    mdg_potential* p = new mdg_potential();
    p->type = POT_LJS;
    p->rcut = rcut;
    const double R2cut = rcut * rcut;
    double rVr2 = rVr * rVr;
    double aVr2 = R2cut / rVr2 - X2min;
    double aLJ3 = (rVr2 / R2cut) * (rVr2 / R2cut) * (rVr2 / R2cut);
    double bLJ2 = (aLJ3 - 0.5) * aVr2 * rVr2 / R2cut;
    double aLJ = (aLJ3 - 1.0 + 2.0 * bLJ2) * aLJ3 / (aVr2 * aVr2);
    double bLJ = -(aLJ3 - 1.0 + 3.0 * bLJ2) * aLJ3 / (aVr2 * aVr2 * aVr2);
    p->ljs_rVr2 = rVr2;
    p->ljs_rVr1 = 1.0 / rVr2;
    p->ljs_aLJ = aLJ;
    p->ljs_bLJ = bLJ;
    p->ljs_aLJ3 = 3.0 * aLJ;
    p->ljs_bLJ2 = 2.0 * bLJ;
    p->ljs_aVr2 = -48.0 * aVr / rVr2;
    p->ljs_aVr = 2.0 * aVr;
    *out = p;
    return MDG_OK;
}

int mdg_pot_pair_create(double rcut, const double* Vpar, int Nr1, double dr, mdg_potential** out) {
    // Pair::Pair(arrays) (pair.cxx:15-33). The table rides the EAM table
    // layout with zero rho and embedding rows, so the force kernels of a
    // Multi solver that mixes it with EAM pairs use one code path.
    if (!out || !Vpar || Nr1 < 3 || !(dr > 0)) {
        set_error("invalid Pair table");
        return MDG_ERR_INVALID;
    }
    mdg_potential* p = new mdg_potential();
    p->type = POT_TAB;
    p->rcut = rcut;
    p->Nr1 = Nr1;
    p->Nrh1 = 3;
    p->dr = dr;
    p->drh = 1.0;
    p->dr1 = 1.0 / dr;
    p->drh1 = 1.0;
    p->Vpar.assign(Vpar, Vpar + Nr1);
    p->dVpar.assign(Nr1 + 1, 0.0);
    init_spline(p->Vpar.data(), p->dVpar.data(), p->dr1, Nr1, 1);
    // one padding element: the reference reads Vpar[N1 + 1] for N1 = Nr1 - 1
    p->Vpar.push_back(p->Vpar.back());
    p->dVpar[Nr1] = p->dVpar[Nr1 - 1];
    p->Rho.assign(Nr1 + 1, 0.0);
    p->dRho.assign(Nr1 + 1, 0.0);
    p->Femb.assign(4, 0.0);
    p->dFemb.assign(4, 0.0);
    *out = p;
    return MDG_OK;
}

int mdg_pot_pair_create_from_file(const char* path, mdg_potential** out) {
    // Pair::Pair(std::string) (pair.cxx:36-56)
    if (!path || !out) return MDG_ERR_INVALID;
    std::ifstream file(path);
    if (!file.is_open()) {
        set_error(std::string("cannot open Pair file: ") + path);
        return MDG_ERR_IO;
    }
    const double N_a = 6.02214076e+23, Qelectron = 1.602176634e-19;
    const double UnMass = 1e-3 / N_a, UnLeng = 1e-9, UnTime = 1e-12;
    const double UnEnrg = UnMass * (UnLeng / UnTime) * (UnLeng / UnTime);
    std::string line;
    for (int k = 0; k < 4; ++k) std::getline(file, line);
    int Nr1 = 0;
    double dr = 0, rcut = 0;
    file >> Nr1 >> dr >> rcut;
    if (!file || Nr1 < 3) {
        set_error("malformed Pair file header");
        return MDG_ERR_IO;
    }
    dr /= 10;
    rcut /= 10;
    std::vector<double> V(Nr1);
    for (int i = 0; i < Nr1; ++i) {
        file >> V[i];
        V[i] *= Qelectron / (10 * UnEnrg);
    }
    if (!file) {
        set_error("Pair file ended before the table was read");
        return MDG_ERR_IO;
    }
    return mdg_pot_pair_create(rcut, V.data(), Nr1, dr, out);
}

int mdg_pot_destroy(mdg_potential* p) {
    if (!p) return MDG_ERR_INVALID;
    if (p->d_tab64) cudaFree(p->d_tab64);
    if (p->d_tab32) cudaFree(p->d_tab32);
    delete p;
    return MDG_OK;
}

int mdg_pot_rcut(mdg_potential* p, double* rcut) {
    if (!p || !rcut) return MDG_ERR_INVALID;
    *rcut = p->rcut;
    return MDG_OK;
}

int mdg_pot_values(mdg_ctx* ctx, mdg_potential* p, const double* r2, size_t n, double* u) {
    if (!ctx || !p || ((!r2 || !u) && n)) return MDG_ERR_INVALID;
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(ctx->device));
    int rc = pot_upload(p, ctx->device);
    if (rc) return rc;
    PotParams P;
    fill_params(p, P, nullptr, nullptr);  // analytic types read no table
    return pot_eval(P, 0, r2, n, u, nullptr, ctx->stream);
}

int mdg_pot_embedding(mdg_ctx* ctx, mdg_potential* p, const double* rho, size_t n, double* F, double* dF) {
    if (!ctx || !p || ((!rho || !F) && n)) return MDG_ERR_INVALID;
    if (p->type != POT_EAM) {
        set_error("the potential has no embedding table");
        return MDG_ERR_INVALID;
    }
    if (n == 0) return MDG_OK;
    MDG_CUDA(cudaSetDevice(ctx->device));
    int rc = pot_upload(p, ctx->device);
    if (rc) return rc;
    PotParams P;
    fill_params(p, P, nullptr, nullptr);
    return pot_eval(P, 1, rho, n, F, dF, ctx->stream);
}

int mdg_pot_atom(mdg_ctx* ctx, mdg_potential* p, int what, mdg_atom* atom, mdg_atom* neibs, size_t nneibs,
                 const uint64_t* list, size_t count, int half) {
    if (!ctx || !p || !atom || (count && (!list || !neibs))) return MDG_ERR_INVALID;
    if (what < MDG_ATOM_FORCE || what > MDG_ATOM_DENSITY) return MDG_ERR_INVALID;
    if (p->type != POT_LJCUT && p->type != POT_EAM) {
        set_error("per-atom evaluation covers LJsCut and EAM");
        return MDG_ERR_INVALID;
    }
    if (p->type == POT_LJCUT && what == MDG_ATOM_DENSITY) {
        set_error("LJsCut has no density");
        return MDG_ERR_INVALID;
    }
    if (count == 0) return MDG_OK;  // the reference returns on an empty list
    if (count > (size_t)INT32_MAX) {
        set_error("list too long");
        return MDG_ERR_INVALID;
    }
    // records: the atom, then each distinct neighbour once (the atom itself
    // when it is listed and lies in neibs)
    const bool inside = atom >= neibs && atom < neibs + nneibs;
    const size_t self = inside ? (size_t)(atom - neibs) : (size_t)-1;
    std::vector<mdg_atom> recs(1, *atom);
    std::vector<uint32_t> slots(count);
    std::unordered_map<uint64_t, uint32_t> slot_of;
    std::vector<uint64_t> owner(1, self);
    for (size_t k = 0; k < count; ++k) {
        const uint64_t j = list[k];
        if (j >= nneibs) {
            set_error("list entry beyond the neighbour array");
            return MDG_ERR_INVALID;
        }
        if (j == self) {
            slots[k] = 0;
            continue;
        }
        auto it = slot_of.find(j);
        if (it == slot_of.end()) {
            it = slot_of.emplace(j, (uint32_t)recs.size()).first;
            recs.push_back(neibs[j]);
            owner.push_back(j);
        }
        slots[k] = it->second;
    }
    MDG_CUDA(cudaSetDevice(ctx->device));
    int rc = pot_upload(p, ctx->device);
    if (rc) return rc;
    PotParams P;
    fill_params(p, P, nullptr, nullptr);
    uint32_t flags = 0;
    rc = pot_atom(P, what, recs.data(), recs.size(), slots.data(), count, half ? 1 : 0, ctx->stream, &flags);
    if (rc) return rc;
    *atom = recs[0];
    for (size_t s = 1; s < recs.size(); ++s) neibs[owner[s]] = recs[s];
    if (flags & FLAG_TABLE) {
        set_error("EAM embedding density outside the table (the reference's extrapolation was used)");
        return MDG_ERR_RANGE;
    }
    return MDG_OK;
}

int mdg_grid_build(mdg_system* sys, int32_t ints[9], double dbls[3]) {
    if (!sys || !ints || !dbls) return MDG_ERR_INVALID;
    if (sys->n == 0) {
        // Grid::initialize_empty (grid.cxx:26-34)
        for (int a = 0; a < 3; ++a) {
            ints[a] = 1;
            ints[3 + a] = 1;
            ints[6 + a] = 0;
            dbls[a] = sys->dom.bmax[a] - sys->dom.bmin[a];
        }
        return MDG_OK;
    }
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    GridParams g;
    int rc = grid_build_only(sys, &g);
    if (rc) return rc;
    for (int a = 0; a < 3; ++a) {
        ints[a] = g.dom_n[a];
        ints[3 + a] = g.offset[a];
        ints[6 + a] = g.num[a];
        dbls[a] = g.cs[a];
    }
    return MDG_OK;
}

// ---- solvers ----------------------------------------------------------------
static void set_stages(mdg_solver* s, int type, bool first) {
    if (type == POT_TAB || type == POT_LJS) type = POT_LJCUT;  // all potential::type::pair
    if (first) {
        if (type == 1) {
            s->nstages = 1;
            s->stages[0] = 1;
        } else if (type == 2) {
            s->nstages = 2;
            s->stages[0] = 0;
            s->stages[1] = 1;
        }
    } else if (type == 2 && s->nstages == 1) {
        s->nstages = 2;
        s->stages[0] = 0;
        s->stages[1] = 1;
    }
}

int mdg_solver_single(mdg_potential* pot, int periodic, mdg_solver** out) {
    if (!pot || !out) return MDG_ERR_INVALID;
    mdg_solver_ext* e = new mdg_solver_ext();
    e->s.multi = 0;
    e->s.nkinds = 1;
    e->s.periodic = periodic ? 1 : 0;
    e->s.pot[0][0] = pot;
    set_stages(&e->s, pot->type, true);
    *out = &e->s;
    return MDG_OK;
}

int mdg_solver_multi(int nkinds, int periodic, mdg_solver** out) {
    if (!out || nkinds < 1 || nkinds > kMaxKinds) {
        set_error("nkinds must be in [1, 4]");
        return MDG_ERR_INVALID;
    }
    mdg_solver_ext* e = new mdg_solver_ext();
    e->s.multi = 1;
    e->s.nkinds = nkinds;
    e->s.periodic = periodic ? 1 : 0;
    *out = &e->s;
    return MDG_OK;
}

int mdg_solver_add_potential(mdg_solver* s, int i, int j, mdg_potential* pot) {
    if (!s || !pot || !s->multi || i < 0 || j < 0 || i >= s->nkinds || j >= s->nkinds) return MDG_ERR_INVALID;
    bool first = s->nstages == 0;
    s->pot[i][j] = pot;
    s->pot[j][i] = pot;
    set_stages(s, pot->type, first);
    ext(s)->version++;
    return MDG_OK;
}

// ---- thermostats ----------------------------------------------------------
static bool langevin_ok(const mdg_langevin* p) {
    return p && p->beta >= 0 && p->temperature >= 0 && p->time_step > 0;
}

int mdg_thermo_langevin_create(const mdg_langevin* params, mdg_thermostat** out) {
    if (!out || !langevin_ok(params)) {
        set_error("Langevin: need beta >= 0, temperature >= 0, time_step > 0");
        return MDG_ERR_INVALID;
    }
    mdg_thermostat* t = new mdg_thermostat();
    t->p = *params;
    *out = t;
    return MDG_OK;
}

int mdg_thermo_langevin_set(mdg_thermostat* t, const mdg_langevin* params) {
    if (!t || t->compound || !langevin_ok(params)) return MDG_ERR_INVALID;
    t->p = *params;
    return MDG_OK;
}

int mdg_thermo_langevin_get(mdg_thermostat* t, mdg_langevin* params) {
    if (!t || t->compound || !params) return MDG_ERR_INVALID;
    *params = t->p;
    return MDG_OK;
}

int mdg_thermo_compound_create(mdg_thermostat** out) {
    if (!out) return MDG_ERR_INVALID;
    mdg_thermostat* t = new mdg_thermostat();
    t->compound = 1;
    *out = t;
    return MDG_OK;
}

int mdg_thermo_compound_add(mdg_thermostat* c, mdg_thermostat* part) {
    if (!c || !part || !c->compound || part == c) return MDG_ERR_INVALID;
    c->parts.push_back(part);
    return MDG_OK;
}

int mdg_thermo_destroy(mdg_thermostat* t) {
    if (!t) return MDG_ERR_INVALID;
    delete t;
    return MDG_OK;
}

// Langevin terms of a thermostat tree in application order.
static int thermo_flatten(const mdg_thermostat* t, ThermoDev& out, int depth) {
    if (depth > 16) {
        set_error("thermostat compound nests too deep");
        return MDG_ERR_INVALID;
    }
    if (!t->compound) {
        if (out.n >= kMaxThermo) {
            set_error("more than 8 Langevin terms in one thermostat");
            return MDG_ERR_INVALID;
        }
        const mdg_langevin& p = t->p;
        LangevinTerm& L = out.t[out.n++];
        L.beta = p.beta;
        // sigma = sqrt(2 beta Kb T / dt) (langevin.cxx:24), Kb of thermostat/base.h:10
        L.sigma = std::sqrt(2.0 * p.beta * 0.008314462175 * p.temperature / p.time_step);
        for (int k = 0; k < 3; ++k) {
            L.heat[k] = (double)p.heat[k];
            L.U[k] = p.U[k];
        }
        L.xmin = p.xmin;
        L.xmax = p.xmax;
        L.seed = p.seed;
        return MDG_OK;
    }
    for (const mdg_thermostat* q : t->parts) {
        int rc = thermo_flatten(q, out, depth + 1);
        if (rc) return rc;
    }
    return MDG_OK;
}

int mdg_solver_set_thermostat(mdg_solver* s, mdg_thermostat* t) {
    if (!s) return MDG_ERR_INVALID;
    s->thermo = t;
    ext(s)->version++;  // captured graphs gain or lose the thermostat pass
    return MDG_OK;
}

static int thermo_sync(mdg_solver* s) {
    if (!s->thermo) return MDG_OK;
    mdg_solver_ext* e = ext(s);
    ThermoDev h;
    memset(&h, 0, sizeof(h));
    int rc = thermo_flatten(s->thermo, h, 0);
    if (rc) return rc;
    if (e->d.th_valid && memcmp(&h, &e->d.th_host, sizeof(h)) == 0) return MDG_OK;
    MDG_CUDA(cudaMemcpy(&blob_of(e->d)->th, &h, sizeof(h), cudaMemcpyHostToDevice));
    e->d.th_host = h;
    e->d.th_valid = 1;
    return MDG_OK;
}

int mdg_system_set_shape(mdg_system* sys, int what, int value) {
    if (!sys || what < 0 || what > 2) return MDG_ERR_INVALID;
    static const int ok[3][4] = {{0, 2, 4, 8}, {0, 3, 4, 8}, {0, 3, 4, 5}};
    bool valid = false;
    for (int v : ok[what]) valid = valid || v == value;
    if (!valid) {
        set_error("unsupported launch shape value");
        return MDG_ERR_INVALID;
    }
    sys->shape[what] = value;
    return MDG_OK;
}

int mdg_system_get_shape(mdg_system* sys, int what, int* value) {
    if (!sys || !value || what < 0 || what > 2) return MDG_ERR_INVALID;
    *value = sys->shape[what];
    return MDG_OK;
}

int mdg_system_thermo_calls(mdg_system* sys, uint32_t* calls) {
    if (!sys || !calls) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    MDG_CUDA(cudaMemcpyAsync(calls, &sys->dstat->therm_calls, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             sys->ctx->stream));
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

int mdg_system_set_thermo_calls(mdg_system* sys, uint32_t calls) {
    if (!sys) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    sys->hstat->therm_calls = calls;
    MDG_CUDA(cudaMemcpyAsync(&sys->dstat->therm_calls, &sys->hstat->therm_calls, sizeof(uint32_t),
                             cudaMemcpyHostToDevice, sys->ctx->stream));
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

int mdg_solver_destroy(mdg_solver* s) {
    if (!s) return MDG_ERR_INVALID;
    mdg_solver_ext* e = ext(s);
    if (e->d.dev) cudaFree(e->d.dev);
    delete e;
    return MDG_OK;
}

int mdg_solver_num_stages(mdg_solver* s, int* n) {
    if (!s || !n) return MDG_ERR_INVALID;
    *n = s->nstages;
    return MDG_OK;
}

int mdg_solver_set_precision(mdg_solver* s, int precision) {
    if (!s || (precision != MDG_PREC_FP64 && precision != MDG_PREC_MIXED)) return MDG_ERR_INVALID;
    s->precision = precision;
    return MDG_OK;
}

// After steps, the outputs each step's prepare clears (Ep and V; Em for EAM
// and for Multi, multi.cxx:51-63) are stale until read or recomputed.
static void mark_stepped(mdg_solver* s, mdg_system* sys, const PotSet& ps) {
    sys->stale_out |= STALE_EP_V | ((ps.any_eam || s->multi) ? STALE_EM : 0);
}

// The step's second half-kick rides in the force pass for the mixed form
// without a thermostat (the thermostat adds its forces after that pass):
// returns the dt to hand to the last stage, 0 when a kick pass follows.
static double fused_kick(mdg_solver* s, int prec, double dt) {
    return prec == MDG_PREC_MIXED && !s->thermo ? dt : 0.0;
}

// Whether a mixed step loop starts each next step inside the force pass
// (k_force_step): the mixed EAM form without a thermostat, whose second
// half-kick already runs there (the EAM force pass reads its neighbours only
// through the density pass's copies, so it can move atoms).
static bool starts_next_step(mdg_solver* s, const PotSet& ps, int prec) {
    return prec == MDG_PREC_MIXED && !s->thermo && ps.any_eam;
}

// The stages of a loop step whose force pass may start the next step
// (launch_forces_step; sys->dcounter holds the steps left, this one
// included): the density pass where the solver has one, then the force pass.
static int step_stages_next(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt) {
    for (int q = 0; q < s->nstages - 1; ++q) {
        cudaEvent_t t0 = timer_begin(sys->ctx);
        int rc = s->stages[q] == 0 ? launch_density_rec(sys, ext(s)->d.dev, ps)
                                   : launch_stage(sys, ext(s)->d.dev, ps, MDG_PREC_MIXED, s->stages[q], nullptr, 0.0);
        timer_end(sys->ctx, s->stages[q] == 0 ? MDG_TIME_DENSITY : MDG_TIME_FORCES, t0);
        if (rc) return rc;
    }
    cudaEvent_t t0 = timer_begin(sys->ctx);
    int rc = launch_forces_step(sys, ext(s)->d.dev, ps, dt, sys->dcounter);
    timer_end(sys->ctx, MDG_TIME_FORCES, t0);
    if (rc) return rc;
    sys->force_prec = MDG_PREC_MIXED;
    return MDG_OK;
}

// The step's stages, the last one carrying the fused kick where it applies,
// then the kick pass where it does not.
static int step_stages(mdg_solver* s, mdg_system* sys, const PotSet& ps, int prec, double dt) {
    const double fk = fused_kick(s, prec, dt);
    if (sys->half) {
        // half lists accumulate both sides of a pair: prepare's clear first
        int rc = launch_zero(sys, ps.any_eam || s->multi);
        if (rc) return rc;
    }
    for (int q = 0; q < s->nstages; ++q) {
        cudaEvent_t t0 = timer_begin(sys->ctx);
        int rc = launch_stage(sys, ext(s)->d.dev, ps, prec, s->stages[q], thermo_of(s),
                              q == s->nstages - 1 ? fk : 0.0);
        timer_end(sys->ctx, s->stages[q] == 0 ? MDG_TIME_DENSITY : MDG_TIME_FORCES, t0);
        if (rc) return rc;
    }
    sys->force_prec = prec;
    if (fk > 0.0) return MDG_OK;
    cudaEvent_t t0 = timer_begin(sys->ctx);
    int rc = launch_kick(sys, dt, prec);
    timer_end(sys->ctx, MDG_TIME_KICK, t0);
    return rc;
}

static int check_ready(mdg_solver* s, mdg_system* sys, PotSet* ps, bool need_list = true) {
    if (!s || !sys) return MDG_ERR_INVALID;
    if (s->nstages == 0) {
        set_error("solver has no potential");
        return MDG_ERR_STATE;
    }
    if (sys->have_list && sys->half && sys->n && s->precision == MDG_PREC_MIXED) {
        set_error("the mixed form needs a full Verlet list (half lists run in the FP64 form)");
        return MDG_ERR_STATE;
    }
    if (need_list && !sys->have_list && sys->n) {
        set_error("no Verlet list: call mdg_nlist_update first");
        return MDG_ERR_STATE;
    }
    // The mixed form takes each pair's minimum image. The Periodic boundary's
    // ghost pass (boundary/periodic.cxx:36-102) gives that image only when
    // every periodic box edge is at least 2 rns; in a smaller box the
    // reference keeps a listed pair's raw difference inside rns.
    if (s->precision == MDG_PREC_MIXED && s->periodic && sys->have_list && sys->n) {
        const GridParams& g = sys->grid;
        for (int a = 0; a < g.dim; ++a)
            if (g.periodic[a] && g.size[a] < 2.0 * g.max_rns) {
                set_error("the mixed form needs every periodic box edge to be at least 2 rns (its minimum images "
                          "are the Periodic boundary's only then); use the FP64 form for this box");
                return MDG_ERR_STATE;
            }
    }
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    if (s->multi) {
        for (int i = 0; i < s->nkinds; ++i)
            for (int j = 0; j < s->nkinds; ++j)
                if (!s->pot[i][j]) {
                    set_error("Multi solver: a kind pair has no potential");
                    return MDG_ERR_STATE;
                }
    }
    int rc = potset_build(s, sys, ps);
    if (rc) return rc;
    return thermo_sync(s);
}

static double pot_rcut_of(mdg_solver* s) { return s->multi ? -1.0 : s->pot[0][0]->rcut; }

int mdg_solver_prepare(mdg_solver* s, mdg_system* sys) {
    // Pair::prepare reads no list (pair.cxx:16-29)
    PotSet ps;
    int rc = check_ready(s, sys, &ps, false);
    if (rc) return rc;
    rc = launch_zero(sys, ps.any_eam || s->multi);
    if (rc) return rc;
    rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 0);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

static int stage_impl(mdg_solver* s, mdg_system* sys, const PotSet& ps, int stage, int prec) {
    mdg_solver_ext* e = ext(s);
    int rc = launch_stage(sys, e->d.dev, ps, prec, stage, thermo_of(s));
    if (rc) return rc;
    if (stage == 1) sys->force_prec = prec;
    return MDG_OK;
}

int mdg_solver_charge(mdg_solver* s, mdg_system* sys) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    rc = stage_impl(s, sys, ps, 0, s->precision);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

int mdg_solver_forces(mdg_solver* s, mdg_system* sys) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    rc = stage_impl(s, sys, ps, 1, s->precision);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

int mdg_solver_stages(mdg_solver* s, mdg_system* sys) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    for (int k = 0; k < s->nstages; ++k) {
        rc = stage_impl(s, sys, ps, s->stages[k], s->precision);
        if (rc) return rc;
    }
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

int mdg_solver_virials(mdg_solver* s, mdg_system* sys) {
    // energies/virials are always evaluated in FP64 (measurement); for the
    // mixed form the FP64 densities are computed first
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    // what the last step's prepare cleared, cleared before the virial pass
    rc = settle_outputs(sys);
    if (rc) return rc;
    mdg_solver_ext* e = ext(s);
    if (ps.any_eam && s->precision == MDG_PREC_MIXED) {
        rc = launch_stage(sys, e->d.dev, ps, MDG_PREC_FP64, 0, nullptr);
        if (rc) return rc;
    } else if (ps.any_eam) {
        // F'(nc) of the current densities (the reference recomputes them)
        rc = launch_stage(sys, e->d.dev, ps, MDG_PREC_FP64, 0, nullptr);
        if (rc) return rc;
    }
    rc = launch_virials(sys, e->d.dev, ps);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

// One Verlet step: drift (+ prepare + rebuild test), stages, kick.
static int step_impl(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt) {
    mdg_solver_ext* e = ext(s);
    int prec = s->precision;
    int rc;
    if (sys->force_prec != prec) {
        rc = launch_force_copy(sys, prec == MDG_PREC_FP64);
        if (rc) return rc;
        sys->force_prec = prec;
    }
    rc = launch_drift(sys, dt, prec, pot_rcut_of(s), s->periodic, 1, 1);
    if (rc) return rc;
    mark_stepped(s, sys, ps);
    return step_stages(s, sys, ps, prec, dt);
}

int mdg_verlet_make_step(mdg_solver* s, mdg_system* sys, double dt) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    if (s->precision == MDG_PREC_MIXED) {
        // Pair::prepare's rcut assignment and boundary flags, then the
        // offsets the mixed kernels read
        rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 0);
        if (rc) return rc;
    }
    rc = step_impl(s, sys, ps, dt);
    if (rc) return rc;
    MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
    return MDG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The driver loop as one CUDA graph: a WHILE node whose body is one Verlet
// step, the rebuild test and an IF node holding the whole list rebuild. The
// conditions are set on the device, so a run of any length is one graph
// launch with no host round trip per step.
// ---------------------------------------------------------------------------
namespace mdg {

// After a step's force pass: the rebuild test of this step's positions
// chooses the rebuild; the test of the next step's positions, when the force
// pass already ran that step's drift, becomes the current one.
__global__ void k_rebuild_cond(cudaGraphConditionalHandle h, DevStatus* st) {
    if (threadIdx.x != 0) return;
    unsigned need = st->need_rebuild;
    st->need_rebuild = st->need_next;
    st->need_next = 0;
    if (need) st->pad[0] += 1;  // rebuilds done inside graphs
    cudaGraphSetConditional(h, need ? 1u : 0u);
}

// One step done; continue while steps remain and no rebuild overflowed its
// capacities (the host then grows them and resumes).
__global__ void k_loop_ctrl(cudaGraphConditionalHandle h, unsigned long long* counter, DevStatus* st) {
    if (threadIdx.x != 0) return;
    unsigned long long c = *counter;
    c = c > 0 ? c - 1 : 0;
    *counter = c;
    bool go = c > 0 && !(st->build_flags & FLAG_OVERFLOW);
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// Whether the step loop runs at all: steps to do and no overflowed rebuild
// before it (the host then grows the capacities and relaunches).
__global__ void k_loop_start(cudaGraphConditionalHandle h, const unsigned long long* counter, const DevStatus* st) {
    if (threadIdx.x != 0) return;
    cudaGraphSetConditional(h, (*counter > 0 && !(st->build_flags & FLAG_OVERFLOW)) ? 1u : 0u);
}

__global__ void k_set_counter(unsigned long long* counter, unsigned long long v, DevStatus* st) {
    if (threadIdx.x == 0) {
        *counter = v;
        st->need_rebuild = 0;
        st->need_next = 0;
        st->build_flags = 0;
        st->pad[0] = 0;
    }
}

static void graph_free(mdg_system* sys) {
    if (sys->run_exec) cudaGraphExecDestroy(sys->run_exec);
    if (sys->run_graph) cudaGraphDestroy(sys->run_graph);
    sys->run_exec = nullptr;
    sys->run_graph = nullptr;
}


static int build_run_graph(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt) {
    graph_free(sys);
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    int prec = s->precision;
    if (!sys->dcounter) {
        int rc = sys_malloc(sys, (void**)&sys->dcounter, sizeof(unsigned long long));
        if (rc) return rc;
    }
    if (starts_next_step(s, ps, prec)) {
        int rc = ensure_cutbits(sys);
        if (rc) return rc;
    }
    cudaGraph_t g = nullptr;
    MDG_CUDA(cudaGraphCreate(&g, 0));
    sys->run_graph = g;
    cudaGraphConditionalHandle hloop, hrb, hpre = 0;
    MDG_CUDA(cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault));
    // a handle must belong to a conditional node: only the mixed form has the pre-rebuild
    if (prec == MDG_PREC_MIXED) MDG_CUDA(cudaGraphConditionalHandleCreate(&hpre, g, 0, cudaGraphCondAssignDefault));

    // Prefix: the mixed form prepares rcut and the boundary flags, rebuilds
    // the list when an upload moved atoms past the half skin (the rebuild
    // test on the prepared state), and refreshes the cell offsets — on the
    // device, so a run starts without a host round trip. Then the WHILE
    // node over steps, entered only when steps remain and no rebuild
    // overflowed.
    uint64_t l0 = ctx->launches;
    int pre_kernels = 0;
    cudaGraphNodeParams pp = {};
    cudaGraphNodeParams wp = {};
    {
        MDG_CUDA(cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        int rc0 = 0;
        cudaError_t e = cudaSuccess;
        auto add_cond = [&](cudaGraphNodeParams& np) {
            cudaStreamCaptureStatus cs0;
            cudaGraph_t cg0 = nullptr;
            const cudaGraphNode_t* d0 = nullptr;
            const cudaGraphEdgeData* ed0 = nullptr;
            size_t nd0 = 0;
            cudaGraphNode_t node = nullptr;
            cudaError_t ee = cudaStreamGetCaptureInfo(st, &cs0, nullptr, &cg0, &d0, &ed0, &nd0);
            if (ee == cudaSuccess) ee = cudaGraphAddNode(&node, cg0, d0, ed0, nd0, &np);
            if (ee == cudaSuccess)
                ee = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
            return ee;
        };
        if (prec == MDG_PREC_MIXED) {
            rc0 = launch_drift(sys, 0.0, MDG_PREC_FP64, s->multi ? -1.0 : s->pot[0][0]->rcut, s->periodic, 0, 1);
            if (rc0 == 0) {
                k_rebuild_cond<<<1, 32, 0, st>>>(hpre, sys->dstat);
                ctx->launches++;
                pp.type = cudaGraphNodeTypeConditional;
                pp.conditional.handle = hpre;
                pp.conditional.type = cudaGraphCondTypeIf;
                pp.conditional.size = 1;
                e = add_cond(pp);
            }
            if (rc0 == 0 && e == cudaSuccess) rc0 = launch_offsets(sys);
            // the first step's half-kick and drift (later steps start in the
            // force pass before them)
            if (rc0 == 0 && e == cudaSuccess && starts_next_step(s, ps, prec))
                rc0 = launch_drift_guarded(sys, dt, sys->dcounter, 1);
        }
        if (rc0 == 0 && e == cudaSuccess) {
            k_loop_start<<<1, 32, 0, st>>>(hloop, sys->dcounter, sys->dstat);
            ctx->launches++;
            wp.type = cudaGraphNodeTypeConditional;
            wp.conditional.handle = hloop;
            wp.conditional.type = cudaGraphCondTypeWhile;
            wp.conditional.size = 1;
            e = add_cond(wp);
        }
        cudaGraph_t outp = nullptr;
        cudaError_t ec = cudaStreamEndCapture(st, &outp);
        if (rc0) return rc0;
        if (e != cudaSuccess) return cuda_status(e, "graph prefix node");
        if (ec != cudaSuccess) return cuda_status(ec, "prefix capture");
        pre_kernels = (int)(ctx->launches - l0);
    }
    if (pp.conditional.phGraph_out) {
        MDG_CUDA(cudaStreamBeginCaptureToGraph(st, pp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
        int rc1 = nlist_enqueue(sys);
        if (rc1 == 0) rc1 = launch_trig(sys);
        cudaGraph_t outr = nullptr;
        cudaError_t ec = cudaStreamEndCapture(st, &outr);
        if (rc1) return rc1;
        if (ec != cudaSuccess) return cuda_status(ec, "pre-rebuild capture");
    }
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    MDG_CUDA(cudaGraphConditionalHandleCreate(&hrb, body, 0, cudaGraphCondAssignDefault));

    l0 = ctx->launches;
    MDG_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const bool next = starts_next_step(s, ps, prec);
    int rc = MDG_OK;
    if (next) {
        rc = step_stages_next(s, sys, ps, dt);
    } else {
        rc = launch_drift(sys, dt, prec, s->multi ? -1.0 : s->pot[0][0]->rcut, s->periodic, 1, 1);
        if (rc == 0) rc = step_stages(s, sys, ps, prec, dt);
    }
    if (rc == 0) {
        k_rebuild_cond<<<1, 32, 0, st>>>(hrb, sys->dstat);
        ctx->launches++;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* ed = nullptr;
    size_t nd = 0;
    cudaGraphNodeParams ip = {};
    cudaGraphNode_t inode = nullptr;
    if (rc == 0) {
        cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &ed, &nd);
        if (e == cudaSuccess) {
            ip.type = cudaGraphNodeTypeConditional;
            ip.conditional.handle = hrb;
            ip.conditional.type = cudaGraphCondTypeIf;
            ip.conditional.size = 1;
            e = cudaGraphAddNode(&inode, cg, deps, ed, nd, &ip);
        }
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(st, &inode, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) rc = cuda_status(e, "graph IF node");
    }
    if (rc == 0) {
        k_loop_ctrl<<<1, 32, 0, st>>>(hloop, sys->dcounter, sys->dstat);
        ctx->launches++;
    }
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(st, &out);
    if (rc) return rc;
    if (e2 != cudaSuccess) return cuda_status(e2, "step capture");
    sys->run_step_kernels = (int)(ctx->launches - l0);

    l0 = ctx->launches;
    MDG_CUDA(cudaStreamBeginCaptureToGraph(st, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal));
    rc = nlist_enqueue(sys);
    if (rc == 0) rc = launch_trig(sys);
    // the next step's half-kick and drift, which the force pass left to
    // after the rebuild (none after the last step)
    if (rc == 0 && next) rc = launch_drift_guarded(sys, dt, sys->dcounter, 2);
    e2 = cudaStreamEndCapture(st, &out);
    if (rc) return rc;
    if (e2 != cudaSuccess) return cuda_status(e2, "rebuild capture");
    sys->run_rebuild_kernels = (int)(ctx->launches - l0);
    sys->run_pre_kernels = pre_kernels;
    // counted when run (the pre-rebuild's kernels are counted as one rebuild)
    ctx->launches -= (uint64_t)sys->run_step_kernels + 2 * (uint64_t)sys->run_rebuild_kernels + pre_kernels;
    MDG_CUDA(cudaGraphInstantiate(&sys->run_exec, g, 0));
    return MDG_OK;
}

// Enqueues `left` steps as one graph launch plus the read-back of the
// remaining-step counter and the status words into pinned memory; does not
// wait.
int run_graph_launch(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, long left) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    uint64_t dtbits;
    memcpy(&dtbits, &dt, sizeof(dtbits));
    const uint64_t shapes = (uint64_t)sys->shape[0] | ((uint64_t)sys->shape[1] << 8) | ((uint64_t)sys->shape[2] << 16);
    uint64_t key[4] = {(uint64_t)(uintptr_t)s, dtbits,
                       (uint64_t)s->precision + 2 * (uint64_t)ext(s)->version + (shapes << 40), sys->cap_version};
    if (!sys->run_exec || memcmp(key, sys->run_key, sizeof(key)) != 0) {
        auto t0 = std::chrono::steady_clock::now();
        int rc = build_run_graph(s, sys, ps, dt);
        if (rc) {
            graph_free(sys);
            return rc;
        }
        memcpy(sys->run_key, key, sizeof(key));
        sys->graph_build_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (!sys->hcounter) MDG_CUDA(cudaMallocHost((void**)&sys->hcounter, sizeof(unsigned long long)));
    k_set_counter<<<1, 32, 0, st>>>(sys->dcounter, (unsigned long long)left, sys->dstat);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaGraphLaunch(sys->run_exec, st));
    MDG_CUDA(cudaMemcpyAsync(sys->hcounter, sys->dcounter, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    sys->run_launched = left;
    sys->force_prec = s->precision;  // what later work in stream order will find
    return MDG_OK;
}

// After the stream work of run_graph_launch completed: bookkeeping, and the
// capacity growth (host path) when the last rebuild overflowed. *left gets
// the steps still to run.
int run_graph_finish(mdg_solver* s, mdg_system* sys, long* left) {
    mdg_ctx* ctx = sys->ctx;
    long rem = (long)*sys->hcounter;
    long done = sys->run_launched - rem;
    uint32_t nreb = sys->hstat->pad[0];
    sys->rebuilds += nreb;
    ctx->launches += (uint64_t)sys->run_pre_kernels + (uint64_t)done * sys->run_step_kernels +
                     (uint64_t)nreb * sys->run_rebuild_kernels;
    sys->force_prec = s->precision;
    *left = rem;
    if (sys->hstat->build_flags & FLAG_OVERFLOW) {
        // the last step's rebuild outgrew a capacity: rebuild on the host
        // path, which grows it, then resume
        sys->rebuilds--;
        int rc = nlist_build(sys, -1.0, sys->half);
        if (rc && rc != MDG_ERR_RANGE) return rc;
    }
    return MDG_OK;
}

static int run_graph(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, long steps) {
    long left = steps;
    for (int round = 0; left > 0 && round < 64; ++round) {
        int rc = run_graph_launch(s, sys, ps, dt, left);
        if (rc) return rc;
        MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
        rc = run_graph_finish(s, sys, &left);
        if (rc) return rc;
    }
    return left > 0 ? MDG_ERR_OVERFLOW : MDG_OK;
}

}  // namespace mdg

extern "C" {

}  // extern "C"

namespace mdg {

// Before the graph loop: forces are brought into the solver's arithmetic
// (the graph's own prefix prepares, re-checks the list and refreshes the
// offsets).
static int graph_prologue(mdg_solver* s, mdg_system* sys) {
    int rc;
    if (sys->force_prec != s->precision) {
        rc = launch_force_copy(sys, s->precision == MDG_PREC_FP64);
        if (rc) return rc;
        sys->force_prec = s->precision;
    }
    return MDG_OK;
}

int run_async_begin(mdg_solver* s, mdg_system* sys, double dt, long steps) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    if (sys->ctx->timing || sys->n == 0 || sys->half) {
        set_error("overlapped runs need a non-empty system with full lists and timing off");
        return MDG_ERR_STATE;
    }
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    rc = graph_prologue(s, sys);
    if (rc) return rc;
    sys->run_launched = 0;
    if (steps <= 0) return MDG_OK;
    mark_stepped(s, sys, ps);
    return run_graph_launch(s, sys, ps, dt, steps);
}

// The whole driver of one request, enqueued on the system's stream with no
// host wait: upload, prepare (rcut, boundary flags), the first list build
// (capacities sized on the host from the same atoms), the initial forces,
// then the graph loop. `first_status` receives the device status right after
// the first build (pinned; valid once the stream passes it): a capacity
// overflow there voids the run and the caller repeats it on the checked
// path. Same operations, in the same order on the device, as
// upload + update(-1) + prepare + stages + mdg_run.
int request_begin(mdg_solver* s, mdg_system* sys, const mdg_atom* atoms, double dt, long steps,
                  DevStatus* first_status) {
    if (!s || s->nstages == 0) {
        set_error("solver has no potential");
        return MDG_ERR_STATE;
    }
    if (sys->n == 0 || sys->ctx->timing) {
        set_error("overlapped runs need a non-empty system and timing off");
        return MDG_ERR_STATE;
    }
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    cudaStream_t st = sys->ctx->stream;
    int rc = upload_atoms_enqueue(sys, atoms, sys->n);
    if (rc) return rc;
    rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 0);
    if (rc) return rc;
    rc = nlist_capacity_host(sys, atoms, sys->n, 0);
    if (rc) return rc;
    sys->grid = *sys->hgrid;
    rc = nlist_enqueue(sys);
    if (rc) return rc;
    rc = launch_trig(sys);
    if (rc) return rc;
    sys->have_list = 1;
    sys->dirty = 0;
    sys->rebuilds++;
    MDG_CUDA(cudaMemcpyAsync(first_status, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    PotSet ps;
    rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    if (s->precision == MDG_PREC_MIXED) {
        rc = launch_offsets(sys);
        if (rc) return rc;
    }
    rc = launch_zero(sys, ps.any_eam || s->multi);
    if (rc) return rc;
    rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 0);
    if (rc) return rc;
    for (int k = 0; k < s->nstages; ++k) {
        rc = stage_impl(s, sys, ps, s->stages[k], s->precision);
        if (rc) return rc;
    }
    sys->run_launched = 0;
    if (steps <= 0) return MDG_OK;
    mark_stepped(s, sys, ps);
    return run_graph_launch(s, sys, ps, dt, steps);
}

const PotSet* solver_potsets(mdg_solver* s, PotSet* host) {
    if (host) *host = ext(s)->d.host;
    return ext(s)->d.dev;
}

int run_async_end(mdg_solver* s, mdg_system* sys, double dt, int* relaunched) {
    *relaunched = 0;
    if (sys->run_launched <= 0) return MDG_OK;
    long left = 0;
    int rc = run_graph_finish(s, sys, &left);
    if (rc) return rc;
    if (left <= 0) return MDG_OK;
    PotSet ps;
    rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    rc = run_graph_launch(s, sys, ps, dt, left);
    if (rc) return rc;
    *relaunched = 1;
    return MDG_OK;
}

}  // namespace mdg

// One step from host buffers with transfers overlapped with the step:
// velocities arrive on the I/O stream while the positions-only prepare and
// list test run; positions leave on the I/O stream once the drift has moved them,
// forces once the force stage is done, velocities after the kick; uploads
// and the step run on the engine's stream. A rebuild at the end of the step
// (it wraps positions) waits for the reads of the permuted arrays and sends
// the positions again. Needs page-locked host buffers (the caller's pinned
// memory); otherwise mdg_run_host takes the graph path.
static int run_host_step_body(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, double* pos,
                              double* vel, double* force);

static int run_host_step(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, double* pos, double* vel,
                         double* force) {
    int rc = run_host_step_body(s, sys, ps, dt, pos, vel, force);
    // no transfer into or out of the caller's buffers may outlive the call,
    // on any exit
    cudaError_t e1 = sys->ctx->io_stream ? cudaStreamSynchronize(sys->ctx->io_stream) : cudaSuccess;
    cudaError_t e2 = cudaStreamSynchronize(sys->ctx->stream);
    if (rc == MDG_OK && e1 != cudaSuccess) rc = cuda_status(e1, "one-step host run");
    if (rc == MDG_OK && e2 != cudaSuccess) rc = cuda_status(e2, "one-step host run");
    return rc;
}

static int run_host_step_body(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, double* pos,
                              double* vel, double* force) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    const size_t n = sys->n;
    const size_t vb = n * 3 * sizeof(double);
    if (!ctx->io_stream) MDG_CUDA(cudaStreamCreateWithFlags(&ctx->io_stream, cudaStreamNonBlocking));
    cudaStream_t io = ctx->io_stream;
    if (sys->step_io_bytes < 3 * vb) {
        sys_free(sys, sys->step_io, sys->step_io_bytes);
        sys->step_io = nullptr;
        sys->step_io_bytes = 0;
        int rc = sys_malloc(sys, (void**)&sys->step_io, 3 * vb);
        if (rc) return rc;
        sys->step_io_bytes = 3 * vb;
    }
    for (cudaEvent_t& e : sys->step_ev)
        if (!e) MDG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaEvent_t ev_flag = sys->step_ev[0], ev_drift = sys->step_ev[1], ev_pos_sent = sys->step_ev[2],
                ev_forces = sys->step_ev[3], ev_reads = sys->step_ev[4], ev_io_done = sys->step_ev[5],
                ev_vel_in = sys->step_ev[6];
    double* xp = sys->step_io;
    double* xf = sys->step_io + 3 * n;
    double* xv = sys->step_io + 6 * n;
    const int prec = s->precision;
    const int nb = (int)((n + kBlock - 1) / kBlock);

    // positions in on the engine's stream, velocities on the I/O stream
    // (through the velocity staging slot) while the positions-only prepare
    // and list test run
    int rc = vec_io(sys, pos, RX, 1, 0);
    if (rc) return rc;
    int c = sys->cur;
    MDG_CUDA(cudaMemcpyAsync(xv, vel, vb, cudaMemcpyHostToDevice, io));
    k_vec_in<<<nb, kBlock, 0, io>>>((int)n, sys->slot_of, xv, sys->f64[VX][c], sys->f64[VY][c], sys->f64[VZ][c]);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaEventRecord(ev_vel_in, io));
    if (prec == MDG_PREC_MIXED) {
        // prepare (rcut, boundary flags) with the list test in one pass, and
        // a rebuild first when the uploaded positions left the list's skin
        MDG_CUDA(cudaMemsetAsync(&sys->dstat->need_rebuild, 0, sizeof(uint32_t), st));
        rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 1);
        if (rc) return rc;
        MDG_CUDA(cudaMemcpyAsync(&sys->hstat->need_rebuild, &sys->dstat->need_rebuild, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, st));
        MDG_CUDA(cudaStreamSynchronize(st));
        if (sys->hstat->need_rebuild) {
            MDG_CUDA(cudaStreamWaitEvent(st, ev_vel_in, 0));  // the rebuild permutes the velocities
            rc = nlist_build(sys, -1.0, sys->half);
            if (rc && rc != MDG_ERR_RANGE) return rc;
            c = sys->cur;
        }
        rc = launch_offsets(sys);
        if (rc) return rc;
    }
    MDG_CUDA(cudaStreamWaitEvent(st, ev_vel_in, 0));
    if (sys->force_prec != prec) {
        rc = launch_force_copy(sys, prec == MDG_PREC_FP64);
        if (rc) return rc;
        sys->force_prec = prec;
    }
    MDG_CUDA(cudaMemsetAsync(&sys->dstat->need_rebuild, 0, sizeof(uint32_t), st));
    rc = launch_drift(sys, dt, prec, pot_rcut_of(s), s->periodic, 1, 1);
    if (rc) return rc;
    MDG_CUDA(cudaMemcpyAsync(&sys->hstat->need_rebuild, &sys->dstat->need_rebuild, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaEventRecord(ev_flag, st));
    MDG_CUDA(cudaEventRecord(ev_drift, st));
    // positions are final for this step (a rebuild below may wrap them)
    MDG_CUDA(cudaStreamWaitEvent(io, ev_drift, 0));
    k_vec_out<<<nb, kBlock, 0, io>>>((int)n, sys->slot_of, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c], xp);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(pos, xp, vb, cudaMemcpyDeviceToHost, io));
    MDG_CUDA(cudaEventRecord(ev_pos_sent, io));
    const double fk = fused_kick(s, prec, dt);
    for (int q = 0; q < s->nstages; ++q) {
        rc = launch_stage(sys, ext(s)->d.dev, ps, prec, s->stages[q], thermo_of(s),
                          q == s->nstages - 1 ? fk : 0.0);
        if (rc) return rc;
    }
    sys->force_prec = prec;
    if (force) {
        MDG_CUDA(cudaEventRecord(ev_forces, st));
        MDG_CUDA(cudaStreamWaitEvent(io, ev_forces, 0));
        if (prec == MDG_PREC_MIXED)
            k_vec_out32<<<nb, kBlock, 0, io>>>((int)n, sys->slot_of, sys->f32[0][c], sys->f32[1][c], sys->f32[2][c], xf);
        else
            k_vec_out<<<nb, kBlock, 0, io>>>((int)n, sys->slot_of, sys->f64[FX][c], sys->f64[FY][c], sys->f64[FZ][c], xf);
        MDG_LAUNCHED(ctx);
    }
    // the I/O stream's reads of the permuted arrays end here
    MDG_CUDA(cudaEventRecord(ev_reads, io));
    if (force) MDG_CUDA(cudaMemcpyAsync(force, xf, vb, cudaMemcpyDeviceToHost, io));
    MDG_CUDA(cudaEventRecord(ev_io_done, io));
    if (fk == 0.0) {
        rc = launch_kick(sys, dt, prec);
        if (rc) return rc;
    }
    k_vec_out<<<nb, kBlock, 0, st>>>((int)n, sys->slot_of, sys->f64[VX][c], sys->f64[VY][c], sys->f64[VZ][c], xv);
    MDG_LAUNCHED(ctx);
    MDG_CUDA(cudaMemcpyAsync(vel, xv, vb, cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaEventSynchronize(ev_flag));
    if (sys->hstat->need_rebuild) {
        // the rebuild permutes what the I/O stream reads
        MDG_CUDA(cudaStreamWaitEvent(st, ev_reads, 0));
        rc = nlist_build(sys, -1.0, sys->half);
        if (rc && rc != MDG_ERR_RANGE) return rc;
        if (prec == MDG_PREC_MIXED) {
            rc = launch_offsets(sys);
            if (rc) return rc;
        }
        c = sys->cur;
        MDG_CUDA(cudaStreamWaitEvent(st, ev_pos_sent, 0));
        k_vec_out<<<nb, kBlock, 0, st>>>((int)n, sys->slot_of, sys->f64[RX][c], sys->f64[RY][c], sys->f64[RZ][c], xp);
        MDG_LAUNCHED(ctx);
        MDG_CUDA(cudaMemcpyAsync(pos, xp, vb, cudaMemcpyDeviceToHost, st));
    }
    MDG_CUDA(cudaStreamWaitEvent(st, ev_io_done, 0));
    return MDG_OK;
}

static bool page_locked(const void* p) {
    if (!p) return true;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

extern "C" {

namespace mdg {
// The host-driven step loop's bookkeeping where the force pass starts the
// next step: the flags and counter as the graph's k_rebuild_cond and
// k_loop_ctrl leave them.
__global__ void k_need_swap(DevStatus* st) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->need_rebuild = st->need_next;
        st->need_next = 0;
    }
}
__global__ void k_counter_dec(unsigned long long* c) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && *c > 0) *c -= 1;
}
}  // namespace mdg

// The step loop of mdg_run driven from the host (timing on), for a mixed
// solver whose force pass starts the next step: the same passes in the same
// order as the graph (first drift; per step density, force + next drift, and
// after a rebuild the next drift as its own pass), each timed.
static int run_loop_next(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt, long steps, cudaEvent_t ev) {
    mdg_ctx* ctx = sys->ctx;
    cudaStream_t st = ctx->stream;
    if (!sys->dcounter) {
        int rc = sys_malloc(sys, (void**)&sys->dcounter, sizeof(unsigned long long));
        if (rc) return rc;
    }
    {
        int rc = ensure_cutbits(sys);
        if (rc) return rc;
    }
    k_set_counter<<<1, 32, 0, st>>>(sys->dcounter, (unsigned long long)steps, sys->dstat);
    MDG_LAUNCHED(ctx);
    if (sys->force_prec != MDG_PREC_MIXED) {
        int rc = launch_force_copy(sys, 0);
        if (rc) return rc;
        sys->force_prec = MDG_PREC_MIXED;
    }
    {
        cudaEvent_t t0 = timer_begin(ctx);
        int rc = launch_drift_guarded(sys, dt, sys->dcounter, 1);
        timer_end(ctx, MDG_TIME_DRIFT, t0);
        if (rc) return rc;
    }
    for (long k = 0; k < steps; ++k) {
        // this step's rebuild test is final before its stages run
        MDG_CUDA(cudaMemcpyAsync(&sys->hstat->need_rebuild, &sys->dstat->need_rebuild, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, st));
        MDG_CUDA(cudaEventRecord(ev, st));
        int rc = step_stages_next(s, sys, ps, dt);
        if (rc) return rc;
        k_need_swap<<<1, 32, 0, st>>>(sys->dstat);
        MDG_LAUNCHED(ctx);
        MDG_CUDA(cudaEventSynchronize(ev));
        if (sys->hstat->need_rebuild) {
            cudaEvent_t t0 = timer_begin(ctx);
            rc = nlist_build(sys, -1.0, sys->half);
            timer_end(ctx, MDG_TIME_REBUILD, t0);
            if (rc && rc != MDG_ERR_RANGE) return rc;
            t0 = timer_begin(ctx);
            rc = launch_drift_guarded(sys, dt, sys->dcounter, 2);
            timer_end(ctx, MDG_TIME_DRIFT, t0);
            if (rc) return rc;
        }
        k_counter_dec<<<1, 32, 0, st>>>(sys->dcounter);
        MDG_LAUNCHED(ctx);
    }
    return MDG_OK;
}

int mdg_run(mdg_solver* s, mdg_system* sys, double dt, long steps) {
    PotSet ps;
    int rc = check_ready(s, sys, &ps);
    if (rc) return rc;
    if (steps <= 0) return MDG_OK;
    mark_stepped(s, sys, ps);
    if (!sys->ctx->timing && sys->n > 0 && !sys->half) {
        rc = graph_prologue(s, sys);
        if (rc) return rc;
        return run_graph(s, sys, ps, dt, steps);
    }
    cudaStream_t st = sys->ctx->stream;
    cudaEvent_t ev;
    MDG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    int prec = s->precision;
    if (prec == MDG_PREC_MIXED) {
        // prepare once (rcut, boundary flags); rebuild first if that or an
        // upload changed what the list was built from
        rc = launch_drift(sys, 0.0, MDG_PREC_FP64, pot_rcut_of(s), s->periodic, 0, 0);
        if (rc) goto done;
        int need = 0;
        rc = mdg_nlist_decide(sys, &need);
        if (rc) goto done;
        if (need) {
            rc = mdg_nlist_update(sys, -1.0, sys->half);
            if (rc && rc != MDG_ERR_RANGE) goto done;
        }
        rc = launch_offsets(sys);
        if (rc) goto done;
    }
    if (starts_next_step(s, ps, prec) && sys->n > 0) {
        rc = run_loop_next(s, sys, ps, dt, steps, ev);
        if (rc) goto done;
        steps = 0;  // done above
    }
    for (long k = 0; k < steps; ++k) {
        cudaError_t ce = cudaMemsetAsync(&sys->dstat->need_rebuild, 0, sizeof(uint32_t), st);
        if (ce != cudaSuccess) {
            rc = cuda_status(ce, "memset");
            goto done;
        }
        if (sys->force_prec != prec) {
            rc = launch_force_copy(sys, prec == MDG_PREC_FP64);
            if (rc) goto done;
            sys->force_prec = prec;
        }
        {
            cudaEvent_t t0 = timer_begin(sys->ctx);
            rc = launch_drift(sys, dt, prec, pot_rcut_of(s), s->periodic, 1, 1);
            timer_end(sys->ctx, MDG_TIME_DRIFT, t0);
        }
        if (rc) goto done;
        // the rebuild flag is final once the drift pass is done
        ce = cudaMemcpyAsync(&sys->hstat->need_rebuild, &sys->dstat->need_rebuild, sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaEventRecord(ev, st);
        if (ce != cudaSuccess) {
            rc = cuda_status(ce, "flag copy");
            goto done;
        }
        rc = step_stages(s, sys, ps, prec, dt);
        if (rc) goto done;
        // overlap: wait for the flag while the force kernels run
        ce = cudaEventSynchronize(ev);
        if (ce != cudaSuccess) {
            rc = cuda_status(ce, "event");
            goto done;
        }
        if (sys->hstat->need_rebuild) {
            cudaEvent_t t0 = timer_begin(sys->ctx);
            rc = nlist_build(sys, -1.0, sys->half);
            timer_end(sys->ctx, MDG_TIME_REBUILD, t0);
            if (rc && rc != MDG_ERR_RANGE) goto done;
            if (prec == MDG_PREC_MIXED) {
                rc = launch_offsets(sys);
                if (rc) goto done;
            }
        }
    }
    {
        cudaError_t ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) rc = cuda_status(ce, "run");
    }
done:
    cudaEventDestroy(ev);
    return rc;
}

int mdg_run_host(mdg_solver* s, mdg_system* sys, double dt, long steps, double* pos, double* vel, double* force) {
    if (!s || !sys || !pos || !vel) return MDG_ERR_INVALID;
    PotSet ps;
    if (steps == 1 && !sys->ctx->timing && sys->n > 0 && !sys->half && check_ready(s, sys, &ps) == MDG_OK &&
        page_locked(pos) && page_locked(vel) && page_locked(force)) {
        MDG_CUDA(cudaSetDevice(sys->ctx->device));
        mark_stepped(s, sys, ps);
        return run_host_step(s, sys, ps, dt, pos, vel, force);
    }
    if (steps > 0 && !sys->ctx->timing && sys->n > 0 && !sys->half && check_ready(s, sys, &ps) == MDG_OK) {
        mark_stepped(s, sys, ps);
        // the whole call in stream order with one wait: uploads, the graph
        // loop, its status read-back, the downloads (the transfer buffer is
        // reused in order, so no transfer waits for another)
        int rc = vec_io(sys, pos, RX, 1, 0);
        if (!rc) rc = vec_io(sys, vel, VX, 1, 0);
        if (!rc) rc = graph_prologue(s, sys);
        if (!rc) rc = run_graph_launch(s, sys, ps, dt, steps);
        if (!rc) rc = vec_io(sys, pos, RX, 0, 0);
        if (!rc) rc = vec_io(sys, vel, VX, 0, 0);
        if (!rc && force) rc = vec_io(sys, force, FX, 0, 0);
        if (rc) return rc;
        MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
        long left = 0;
        rc = run_graph_finish(s, sys, &left);
        if (rc) return rc;
        if (left == 0) return MDG_OK;
        // a rebuild outgrew its capacities (grown now): finish the steps and
        // download again
        rc = run_graph(s, sys, ps, dt, left);
        if (rc) return rc;
        rc = vec_io(sys, pos, RX, 0, 0);
        if (!rc) rc = vec_io(sys, vel, VX, 0, 0);
        if (!rc && force) rc = vec_io(sys, force, FX, 0, 0);
        if (rc) return rc;
        MDG_CUDA(cudaStreamSynchronize(sys->ctx->stream));
        return MDG_OK;
    }
    int rc = mdg_system_set_positions(sys, pos);
    if (rc) return rc;
    rc = mdg_system_set_velocities(sys, vel);
    if (rc) return rc;
    rc = mdg_run(s, sys, dt, steps);
    if (rc && rc != MDG_ERR_RANGE) return rc;
    rc = mdg_system_get_positions(sys, pos);
    if (rc) return rc;
    rc = mdg_system_get_velocities(sys, vel);
    if (rc) return rc;
    if (force) rc = mdg_system_get_forces(sys, force);
    return rc;
}

int mdg_system_measure(mdg_system* sys, mdg_state* out) {
    if (!sys || !out) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    int rc = settle_outputs(sys);
    if (rc) return rc;
    double r[11];
    rc = launch_measure(sys, r);
    if (rc) return rc;
    out->Ep = r[0];
    out->Em = r[1];
    out->virial = r[2];
    out->KE = r[7];
    out->Etot = r[0] + r[1] + r[7];
    out->vcom[0] = r[8];
    out->vcom[1] = r[9];
    out->vcom[2] = r[10];
    return MDG_OK;
}

int mdg_system_flags(mdg_system* sys, uint32_t* flags) {
    if (!sys || !flags) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(sys->ctx->device));
    cudaStream_t st = sys->ctx->stream;
    MDG_CUDA(cudaMemcpyAsync(sys->hstat, sys->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, st));
    MDG_CUDA(cudaStreamSynchronize(st));
    *flags = sys->hstat->flags;
    MDG_CUDA(cudaMemsetAsync(&sys->dstat->flags, 0, sizeof(uint32_t), st));
    MDG_CUDA(cudaStreamSynchronize(st));
    return MDG_OK;
}

}  // extern "C"
