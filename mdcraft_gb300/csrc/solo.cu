// solo.cu — the whole driver loop of one small system in one thread block.
//
// For the serving loop's systems (hundreds to tens of thousands of atoms) a
// step is a few microseconds of work spread over a few SMs, so launching its
// stages as separate kernels (or graph nodes) costs more than the work. Here
// one block owns one system and runs `steps` iterations of the driver loop
// of the reference (test/python/solver/test-EAM.py:158-200: make_step, then
// decide() and update(-1)) with block barriers between the passes:
//   drift + half-skin test -> [EAM density ->] forces -> kick
//   -> if any atom moved half a skin: the rebuild (wrap + bounds, grid,
//      bin count, scan, scatter, in-bin sort, permutation of every field,
//      cell offsets, list build) -> next step.
// Every pass calls the same per-atom (or per-bin) device code as the
// per-stage kernels, in the same order, so a system gives the same bits
// here as through mdg_run. Many systems run at once, one block each, in
// shared launches. Nothing in the loop waits on another block.
#include <cuda_runtime.h>

#include <atomic>

#include "forces_dev.cuh"
#include "integrate_dev.cuh"
#include "mdg_host.h"
#include "nlist_dev.cuh"

namespace mdg {

// Completion record of one system's run, in host-mapped pinned memory: the
// block writes it last, `done` after a system-scope fence.
struct SoloOut {
    unsigned long long left;
    DevStatus st;
    volatile uint32_t done;
    uint32_t pad;
    // GPU clock (%globaltimer, ns): the block starts on the request / has
    // written the result records (service time = end - start)
    unsigned long long t_start, t_end;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct alignas(16) SoloArgs {
    IArgs I;
    FArgs F;
    NbArgs N;
    GatherAll G;
    DomainDev D;
    const PotSet* ps;
    int n;
    double *rx, *ry, *rz;
    const double* rns;
    uint32_t *key, *rank, *src, *bin_count, *bin_start;
    const uint32_t* orig;
    uint32_t* cellp;
    double *Rx, *Ry, *Rz;
    int4 *pos32, *q0;
    float4* o0;
    uint32_t* slot_of;
    const double *saved_rns, *saved_rcut;
    float2* trig;
    GridParams* dgrid;
    long long bin_cap;
    DevStatus* st;
    long long steps;              // steps to run
    uint32_t seq;                 // completion value written to out->done
    int np;
    int setup;                    // 1: load the atoms, build the first list, initial forces
    int any_eam;
    const mdg_atom* atoms_in;     // host-mapped input records (setup)
    uint8_t* bc;
    SoloOut* out;                 // host-mapped: steps left, status, completion
    mdg_atom* atoms_out;          // host-mapped: the result records, caller order
};

constexpr int kSoloMaxAtoms = 65536;

template <int NT>
__device__ __forceinline__ void gather_block(const GatherAll& G, const uint32_t* src, int n) {
    for (int k = threadIdx.x; k < n; k += NT) {
        uint32_t s = src[k];
#pragma unroll
        for (int f = 0; f < 12; ++f) G.a.out[f][k] = G.a.in[f][s];
#pragma unroll
        for (int f = 0; f < 12; ++f) G.b.out[f][k] = G.b.in[f][s];
#pragma unroll
        for (int f = 0; f < 3; ++f) G.fc.out[f][k] = G.fc.in[f][s];
#pragma unroll
        for (int f = 0; f < 2; ++f) G.u.out[f][k] = G.u.in[f][s];
#pragma unroll
        for (int f = 0; f < 2; ++f) G.h.out[f][k] = G.h.in[f][s];
    }
}

template <int NT>
__device__ __forceinline__ void copy_back_block(const GatherAll& G, int n) {
    for (int k = threadIdx.x; k < n; k += NT) {
#pragma unroll
        for (int f = 0; f < 12; ++f) G.a2.out[f][k] = G.a2.in[f][k];
#pragma unroll
        for (int f = 0; f < 12; ++f) G.b2.out[f][k] = G.b2.in[f][k];
#pragma unroll
        for (int f = 0; f < 3; ++f) G.fc2.out[f][k] = G.fc2.in[f][k];
#pragma unroll
        for (int f = 0; f < 2; ++f) G.u2.out[f][k] = G.u2.in[f][k];
#pragma unroll
        for (int f = 0; f < 2; ++f) G.h2.out[f][k] = G.h2.in[f][k];
    }
}

// One rebuild by the whole block (the pipeline of nlist_enqueue + trig).
// Block-uniform result: false when a capacity overflowed (the loop stops and
// the host grows the capacities).
template <int NT>
__device__ __noinline__ bool solo_rebuild(const SoloArgs& S, GridParams& g, double (*red)[NT / 32], uint32_t* scan_sh) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, n = S.n;
    if (t == 0) {
        S.st->max_count = 0;
        S.st->nonuniform = 0;
        S.st->build_flags = 0;
    }
    // wrap + bounds (min/max are exact, so the order of the reduction is free)
    double v7[7] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308,
                    -1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308, 0.0};
    for (int i = t; i < n; i += NT) {
        double v[3];
        wrap_one(S.D, S.rx, S.ry, S.rz, i, v);
        for (int a = 0; a < 3; ++a) {
            v7[a] = fmin(v7[a], v[a]);
            v7[3 + a] = fmax(v7[3 + a], v[a]);
        }
        double q = S.rns[i];
        v7[6] = v7[6] < q ? q : v7[6];
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 7; ++k) {
            double y = __shfl_down_sync(0xffffffffu, v7[k], o);
            v7[k] = k < 3 ? fmin(v7[k], y) : fmax(v7[k], y);
        }
    if (lane == 0)
        for (int k = 0; k < 7; ++k) red[k][w] = v7[k];
    __syncthreads();
    if (t == 0) {
        for (int q = 1; q < NT / 32; ++q)
            for (int k = 0; k < 7; ++k) red[k][0] = k < 3 ? fmin(red[k][0], red[k][q]) : fmax(red[k][0], red[k][q]);
        double lo[3] = {red[0][0], red[1][0], red[2][0]}, hi[3] = {red[3][0], red[4][0], red[5][0]};
        GridParams gg;
        grid_from_bounds(S.D, lo, hi, red[6][0], gg);
        if (gg.empty == 0 && (long long)gg.nbins + 1 > S.bin_cap) {
            gg.empty = -3;
            atomicOr(&S.st->flags, FLAG_OVERFLOW);
            atomicOr(&S.st->build_flags, FLAG_OVERFLOW);
        }
        g = gg;
        *S.dgrid = gg;
    }
    // nonuniform rns (the list's FP32 prefilter needs one rns for all)
    {
        double r0 = S.rns[0];
        for (int i = t; i < n; i += NT)
            if (S.rns[i] != r0) atomicOr(&S.st->nonuniform, 1u);
    }
    __syncthreads();
    if (g.empty) {
        bool ok = g.empty != -3;
        __syncthreads();
        return ok;
    }
    const int nb = g.nbins;
    for (long long b = t; b < S.bin_cap; b += NT) S.bin_count[b] = 0;
    __syncthreads();
    for (int i = t; i < n; i += NT) bin_count_one(g, i, S.rx, S.ry, S.rz, S.key, S.rank, S.bin_count, S.st);
    __syncthreads();
    // exclusive scan: each thread a contiguous chunk of the bins
    {
        const int chunk = (nb + NT - 1) / NT;
        const int b0 = min(t * chunk, nb), b1 = min(b0 + chunk, nb);
        uint32_t sum = 0;
        for (int b = b0; b < b1; ++b) sum += S.bin_count[b];
        uint32_t tot;
        uint32_t off = block_excl_scan(sum, scan_sh, &tot);
        for (int b = b0; b < b1; ++b) {
            uint32_t c = S.bin_count[b];
            S.bin_start[b] = off;
            off += c;
        }
        if (t == 0) S.bin_start[nb] = tot;
    }
    __syncthreads();
    for (int i = t; i < n; i += NT) S.src[S.bin_start[S.key[i]] + S.rank[i]] = (uint32_t)i;
    __syncthreads();
    for (int b = t; b < nb; b += NT) bin_sort_one(b, S.bin_start, S.src, S.orig);
    __syncthreads();
    gather_block<NT>(S.G, S.src, n);
    __syncthreads();
    copy_back_block<NT>(S.G, n);
    __syncthreads();
    for (int i = t; i < n; i += NT)
        cells_one(g, i, S.rx, S.ry, S.rz, S.cellp, S.Rx, S.Ry, S.Rz, S.pos32, S.q0, S.o0, S.orig, S.slot_of, S.F.kind);
    __syncthreads();
    {
        const bool uniform = S.st->nonuniform == 0;
        if (!g.small_box) {
            // a warp per cell, lanes over candidates (the per-stage list
            // build's body); its per-warp state is the launch's dynamic
            // shared memory
            extern __shared__ __align__(16) unsigned char solo_dyn[];
            NbWarpSmem* nbs = reinterpret_cast<NbWarpSmem*>(solo_dyn);
            for (int b = w; b < nb; b += NT / 32) nbuild_cell_warp(S.N, g, b, lane, uniform, nbs[w]);
        } else {
            // a few cells of many atoms: a thread per atom
            for (int i = t; i < n; i += NT) nbuild_atom(S.N, g, (uint32_t)i, uniform);
        }
        __syncthreads();
        // atoms clamped into the grid: their own lists from their unclamped cells
        if (!g.small_box && (S.st->build_flags & FLAG_RANGE))
            for (int i = t; i < n; i += NT)
                if (S.N.o0[i].w == 2.0f) nbuild_atom(S.N, g, (uint32_t)i, uniform);
    }
    __syncthreads();
    for (int i = t; i < n; i += NT) trig_one(i, S.saved_rns, S.saved_rcut, g, S.trig);
    __syncthreads();
    bool ok = !(S.st->build_flags & FLAG_OVERFLOW);
    __syncthreads();
    return ok;
}

// The input records (mdg_system_upload_atoms' scatter) from host memory.
template <int NT>
__device__ __noinline__ void solo_read_atoms(const SoloArgs& S) {
    const GatherAll& G = S.G;
    for (int k = threadIdx.x; k < S.n; k += NT) {
        const mdg_atom& a = S.atoms_in[k];
        const uint32_t s = S.slot_of[k];
        for (int c = 0; c < 3; ++c) {
            G.a2.out[RX + c][s] = a.r[c];
            G.a2.out[VX + c][s] = a.v[c];
            G.a2.out[FX + c][s] = a.f[c];
            G.fc2.out[c][s] = (float)a.f[c];
        }
        G.a2.out[MASS][s] = a.m;
        G.a2.out[RCUT][s] = a.rcut;
        G.a2.out[RNS][s] = a.rns;
        G.b2.out[EP - 12][s] = a.Ep;
        G.b2.out[EM - 12][s] = a.Em;
        G.b2.out[NC - 12][s] = a.nc;
        for (int q = 0; q < 9; ++q) G.b2.out[V0 - 12 + q][s] = a.V[q];
        G.u2.out[1][s] = a.uid;
        G.h2.out[0][s] = a.kind;
        G.h2.out[1][s] = a.tag;
    }
}

// Pair::prepare's output reset (launch_zero) for atom i.
__device__ __forceinline__ void solo_zero_one(const SoloArgs& S, int i) {
    const GatherAll& G = S.G;
    if (G.h.in[1][i] == 0) return;
    G.a2.out[FX][i] = 0.0;
    G.a2.out[FY][i] = 0.0;
    G.a2.out[FZ][i] = 0.0;
    G.b2.out[EP - 12][i] = 0.0;
    for (int k = 0; k < 9; ++k) G.b2.out[V0 - 12 + k][i] = 0.0;
    if (S.any_eam) {
        G.b2.out[EM - 12][i] = 0.0;
        G.b2.out[NC - 12][i] = 0.0;
    }
}

// The force stages; with KICK the second half-kick rides in the force body
// (the step loop), without it the forces alone (the set-up's initial forces).
template <bool EAM, bool KICK, int NT>
__device__ __forceinline__ void solo_stages(const SoloArgs& S) {
    const int t = threadIdx.x, n = S.n;
    if (EAM) {
        for (int i = t; i < n; i += NT) density_mixed_one<false>(S.F, S.ps, i);
        __syncthreads();
        for (int i = t; i < n; i += NT) eam_mixed_one<false, KICK>(S.F, S.ps, i);
    } else {
        for (int i = t; i < n; i += NT) lj_mixed_one<false, KICK>(S.F, S.ps, i);
    }
}

// The set-up of a fresh system, in the order of the host calls it replaces
// (upload, prepare, update(-1), offsets, prepare, stages). False when the
// first list outgrew the capacities sized on the host.
template <bool EAM, int NT>
__device__ __noinline__ bool solo_setup(const SoloArgs& S, GridParams& g, double (*red)[NT / 32], uint32_t* scan_sh) {
    const int t = threadIdx.x, n = S.n;
    // the fresh system's buffers (what system_alloc clears on a stream)
    for (int k = t; k < S.np; k += NT) {
        S.G.u2.out[0][k] = (uint32_t)k;  // caller index of slot k
        S.slot_of[k] = (uint32_t)k;
        S.N.ncnt[k] = 0;
        S.bc[k] = 0;
        S.trig[k] = make_float2(0.0f, 0.0f);
        S.Rx[k] = 0.0;
        S.Ry[k] = 0.0;
        S.Rz[k] = 0.0;
        for (int q = 0; q < kMaxKinds; ++q) S.F.Fp64[(size_t)q * S.np + k] = 0.0;
    }
    if (t == 0) memset(S.st, 0, sizeof(DevStatus));
    __syncthreads();
    solo_read_atoms<NT>(S);
    __syncthreads();
    for (int i = t; i < n; i += NT) drift64_one(S.I, i, 0, 0);
    __syncthreads();
    if (!solo_rebuild<NT>(S, g, red, scan_sh)) return false;
    for (int i = t; i < n; i += NT)
        S.pos32[i] = make_int4(off_encode(S.rx[i] - S.Rx[i], g.inv_u[0]), off_encode(S.ry[i] - S.Ry[i], g.inv_u[1]),
                               off_encode(S.rz[i] - S.Rz[i], g.inv_u[2]), S.F.kind[i] & 3);
    for (int i = t; i < n; i += NT) solo_zero_one(S, i);
    __syncthreads();
    for (int i = t; i < n; i += NT) drift64_one(S.I, i, 0, 0);
    __syncthreads();
    solo_stages<EAM, false, NT>(S);
    __syncthreads();
    return true;
}

// The result records (mdg_system_download_atoms' layout) straight into host
// memory; mixed forces are widened to FP64 as the download does.
template <int NT>
__device__ __noinline__ void solo_write_atoms(const SoloArgs& S) {
    const GatherAll& G = S.G;
    for (int k = threadIdx.x; k < S.n; k += NT) {
        const uint32_t s = S.slot_of[k];
        mdg_atom a;
        const bool live = G.h.in[1][s] != 0;  // tag
        for (int c = 0; c < 3; ++c) {
            a.r[c] = G.a.in[RX + c][s];
            a.v[c] = G.a.in[VX + c][s];
            a.f[c] = live ? (double)G.fc.in[c][s] : G.a.in[FX + c][s];
        }
        a.m = G.a.in[MASS][s];
        a.rcut = G.a.in[RCUT][s];
        a.rns = G.a.in[RNS][s];
        a.Ep = G.b.in[EP - 12][s];
        a.Em = G.b.in[EM - 12][s];
        a.nc = G.b.in[NC - 12][s];
        for (int q = 0; q < 9; ++q) a.V[q] = G.b.in[V0 - 12 + q][s];
        a.uid = G.u.in[1][s];
        a.kind = G.h.in[0][s];
        a.tag = G.h.in[1][s];
        a.bc = S.bc[s];
        a._pad[0] = a._pad[1] = a._pad[2] = 0;
        S.atoms_out[k] = a;
    }
}

// One request by the whole block: set-up, the loop, the result records and
// the completion record (last, after a system-scope fence).
template <bool EAM, int NT>
__device__ void solo_run(SoloArgs& S, GridParams& g, double (*red)[NT / 32], uint32_t* scan_sh) {
    const int t = threadIdx.x, n = S.n;
    long long left = S.steps;
    uint32_t rebuilds = 0;
    bool ok = true;
    unsigned long long t_start = 0;
    if (t == 0) t_start = global_ns();
    if (S.setup) ok = solo_setup<EAM, NT>(S, g, red, scan_sh);
    if (t == 0) {
        S.st->need_rebuild = 0;
        S.st->build_flags = 0;
    }
    while (ok && left > 0) {
        bool need = false;
        for (int i = t; i < n; i += NT) need |= drift_mixed_one(S.I, i);
        const int any = __syncthreads_or(need);
        solo_stages<EAM, true, NT>(S);
        __syncthreads();
        --left;
        if (any) {
            ++rebuilds;
            ok = solo_rebuild<NT>(S, g, red, scan_sh);
        }
    }
    if (ok && left == 0) solo_write_atoms<NT>(S);
    __syncthreads();
    if (t == 0) {
        S.st->need_rebuild = 0;
        S.st->pad[0] = rebuilds;
        S.st->pad[1] = ok ? 0u : 1u;  // 1: a list outgrew its capacities; the run is void
        S.out->left = (unsigned long long)left;
        S.out->st = *S.st;
        S.out->t_start = t_start;
        S.out->t_end = global_ns();
        __threadfence_system();
        S.out->done = S.seq;
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t ld_acquire_sys(const volatile uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Persistent consumer of the request queue: each block claims the next
// published entry, runs that request, and claims again; a block that finds
// no entry for `idle_limit` polls (about a microsecond apart), or sees
// `stop`, exits. Every wait is bounded.
template <int NT>
__global__ void __launch_bounds__(NT, 1) k_solo_persistent(const SoloArgs* __restrict__ desc, SoloQueue* q,
                                                           uint32_t* head, int idle_limit, int gen) {
    __shared__ __align__(16) SoloArgs S;
    __shared__ GridParams g;
    __shared__ double red[7][NT / 32];
    __shared__ uint32_t scan_sh[32];
    __shared__ int s_rec;
    // liveness for the host (which set 1 before the launch), so that it tops
    // up the kernel with a further launch when blocks have gone idle and
    // exited while requests wait
    if (threadIdx.x == 0) q->live[gen][blockIdx.x] = 1u;
    for (;;) {
        if (threadIdx.x == 0) {
            int rec = -1;
            for (int it = 0; it < idle_limit; ++it) {
                const uint32_t tl = ld_acquire_sys(&q->tail);
                const uint32_t h = *(volatile uint32_t*)head;
                if (h < tl) {
                    if (atomicCAS(head, h, h + 1) == h) {
                        rec = ((volatile int*)q->ring)[h % kSoloRing];
                        break;
                    }
                    continue;
                }
                if (q->stop) break;
                __nanosleep(1000);
            }
            s_rec = rec;
        }
        __syncthreads();
        const int rec = s_rec;
        if (rec < 0) break;
        if (threadIdx.x == 0) q->live[gen][blockIdx.x] = 2u;  // 2: running a request
        {
            const int4* src = reinterpret_cast<const int4*>(desc + rec);
            int4* dst = reinterpret_cast<int4*>(&S);
            for (int k = threadIdx.x; k < (int)(sizeof(SoloArgs) / sizeof(int4)); k += NT) dst[k] = src[k];
        }
        __syncthreads();
        if (S.any_eam) solo_run<true, NT>(S, g, red, scan_sh);
        else solo_run<false, NT>(S, g, red, scan_sh);
        if (threadIdx.x == 0) q->live[gen][blockIdx.x] = 1u;  // 1: waiting for the next entry
    }
    if (threadIdx.x == 0) {
        __threadfence_system();
        q->live[gen][blockIdx.x] = 0u;
    }
}

int solo_eligible(const mdg_solver* s, const mdg_system* sys) {
    if (s->precision != MDG_PREC_MIXED || s->multi || s->nstages < 1 || s->thermo) return 0;
    // the fused loop carries the LJsCut and EAM bodies only
    if (!s->pot[0][0] || (s->pot[0][0]->type != POT_LJCUT && s->pot[0][0]->type != POT_EAM)) return 0;
    if (sys->n == 0 || sys->n > (size_t)kSoloMaxAtoms || sys->half || !sys->cap_ready || sys->ctx->timing) return 0;
    return 1;
}

void solo_fill(void* args, mdg_system* sys, const PotSet* dps, int any_eam, double pot_rcut, int periodic,
               double dt, long steps, const void* atoms_in_dev, void* out_dev, void* atoms_out_dev, uint32_t seq) {
    SoloArgs& S = *reinterpret_cast<SoloArgs*>(args);
    memset(&S, 0, sizeof(S));
    S.I = integrator_args(sys, dt);
    S.I.pot_rcut = pot_rcut;
    S.I.periodic_boundary = periodic;
    S.setup = 1;
    S.seq = seq;
    S.np = (int)sys->np;
    S.any_eam = any_eam;
    S.atoms_in = reinterpret_cast<const mdg_atom*>(atoms_in_dev);
    S.F = force_args(sys);
    S.F.kick_hdt = 0.5f * (float)dt;  // the step loop's second half-kick, in the force body
    S.N = nb_args(sys);
    S.G = gather_sets(sys);
    S.D = domain_of(sys);
    S.ps = dps;
    S.n = (int)sys->n;
    const int c = sys->cur;
    S.rx = sys->f64[RX][c];
    S.ry = sys->f64[RY][c];
    S.rz = sys->f64[RZ][c];
    S.rns = sys->f64[RNS][c];
    S.key = sys->key;
    S.rank = sys->rank;
    S.src = sys->src;
    S.bin_count = sys->bin_count;
    S.bin_start = sys->bin_start;
    S.orig = sys->u32[ORIG][c];
    S.cellp = sys->cellp;
    S.Rx = sys->Rc[0];
    S.Ry = sys->Rc[1];
    S.Rz = sys->Rc[2];
    S.pos32 = sys->pos32;
    S.q0 = sys->q0;
    S.o0 = sys->o0;
    S.slot_of = sys->slot_of;
    S.saved_rns = sys->saved_rns;
    S.saved_rcut = sys->saved_rcut;
    S.trig = sys->trig32;
    S.dgrid = sys->dgrid;
    S.bin_cap = (long long)sys->bin_cap;
    S.st = sys->dstat;
    S.steps = steps;
    S.bc = sys->bc;
    S.out = reinterpret_cast<SoloOut*>(out_dev);
    S.atoms_out = reinterpret_cast<mdg_atom*>(atoms_out_dev);
}

size_t solo_args_bytes() { return sizeof(SoloArgs); }
static_assert(sizeof(SoloArgs) % 16 == 0, "argument records are copied as 16-byte words");
size_t solo_out_bytes() { return sizeof(SoloOut); }

int solo_out_read(const void* out_host, uint32_t* done, unsigned long long* left, DevStatus* st,
                  double* service_s) {
    const SoloOut* o = reinterpret_cast<const SoloOut*>(out_host);
    *done = __atomic_load_n(const_cast<const uint32_t*>(&o->done), __ATOMIC_ACQUIRE);
    if (left) *left = o->left;
    if (st) *st = o->st;
    if (service_s) *service_s = o->t_end > o->t_start ? (double)(o->t_end - o->t_start) * 1e-9 : 0.0;
    return MDG_OK;
}

// Dynamic shared memory of a launch: the list build's state, one per warp.
static size_t solo_dyn_bytes(int threads) { return (size_t)(threads / 32) * sizeof(NbWarpSmem); }

// The launch's dynamic shared memory exceeds the default 48 KB at 1024
// threads; the attribute is per device, so it is set once per device.
template <int NT>
static cudaError_t solo_prepare_attr() {
    static std::atomic<uint64_t> done{0};  // bit d: set on device d (devices 0..63)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (done.load() & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(k_solo_persistent<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)solo_dyn_bytes(NT));
    if (e == cudaSuccess && bit) done.fetch_or(bit);
    return e;
}

int solo_persistent_launch(cudaStream_t stream, int threads, int blocks, const void* desc_dev, SoloQueue* q_dev,
                           uint32_t* head, int idle_limit, int gen) {
    const SoloArgs* d = reinterpret_cast<const SoloArgs*>(desc_dev);
    if (blocks <= 0) return MDG_OK;
    if (blocks > kSoloMaxBlocks || gen < 0 || gen >= kSoloGens) return MDG_ERR_INVALID;
    const size_t dyn = solo_dyn_bytes(threads);
    if (threads == 640) {
        MDG_CUDA(solo_prepare_attr<640>());
        k_solo_persistent<640><<<blocks, 640, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    } else if (threads == 768) {
        MDG_CUDA(solo_prepare_attr<768>());
        k_solo_persistent<768><<<blocks, 768, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    } else if (threads == 896) {
        MDG_CUDA(solo_prepare_attr<896>());
        k_solo_persistent<896><<<blocks, 896, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    } else if (threads == 256) {
        MDG_CUDA(solo_prepare_attr<256>());
        k_solo_persistent<256><<<blocks, 256, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    } else if (threads == 1024) {
        MDG_CUDA(solo_prepare_attr<1024>());
        k_solo_persistent<1024><<<blocks, 1024, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    } else {
        MDG_CUDA(solo_prepare_attr<512>());
        k_solo_persistent<512><<<blocks, 512, dyn, stream>>>(d, q_dev, head, idle_limit, gen);
    }
    MDG_CUDA(cudaGetLastError());
    return MDG_OK;
}

int solo_graph_launch(SoloGraph& G, cudaStream_t stream, int threads, int blocks, const void* desc_dev,
                      SoloQueue* q_dev, uint32_t* head, int idle_limit, int gen) {
    if (blocks <= 0) return MDG_OK;
    if (blocks > kSoloMaxBlocks || gen < 0 || gen >= kSoloGens) return MDG_ERR_INVALID;
    if (!G.exec) {
        // the kernel's shared-memory attribute is set before the capture (it
        // is not a stream operation)
        int per_sm = 0;
        int rc = solo_blocks_per_sm(threads, &per_sm);
        if (rc) return rc;
        MDG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        rc = solo_persistent_launch(stream, threads, blocks, desc_dev, q_dev, head, idle_limit, gen);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (rc != MDG_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc != MDG_OK ? rc : cuda_status(e, "persistent kernel capture");
        }
        cudaGraphNode_t node = nullptr;
        size_t nn = 1;
        e = cudaGraphGetNodes(g, &node, &nn);
        if (e == cudaSuccess && nn != 1) {
            cudaGraphDestroy(g);
            set_error("persistent kernel capture: expected one kernel node");
            return MDG_ERR_CUDA;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&G.exec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            G.exec = nullptr;
            return cuda_status(e, "persistent kernel graph");
        }
        G.graph = g;
        G.node = node;
    } else {
        cudaKernelNodeParams p;
        MDG_CUDA(cudaGraphKernelNodeGetParams(G.node, &p));
        p.gridDim = dim3((unsigned)blocks, 1, 1);
        MDG_CUDA(cudaGraphExecKernelNodeSetParams(G.exec, G.node, &p));
    }
    MDG_CUDA(cudaGraphLaunch(G.exec, stream));
    return MDG_OK;
}

void solo_graph_destroy(SoloGraph& G) {
    if (G.exec) cudaGraphExecDestroy(G.exec);
    if (G.graph) cudaGraphDestroy(G.graph);
    G = SoloGraph();
}

int solo_blocks_per_sm(int threads, int* blocks) {
    cudaError_t e;
    const size_t dyn = solo_dyn_bytes(threads);
    if (threads == 640) {
        MDG_CUDA(solo_prepare_attr<640>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<640>, 640, dyn);
    } else if (threads == 768) {
        MDG_CUDA(solo_prepare_attr<768>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<768>, 768, dyn);
    } else if (threads == 896) {
        MDG_CUDA(solo_prepare_attr<896>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<896>, 896, dyn);
    } else if (threads == 256) {
        MDG_CUDA(solo_prepare_attr<256>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<256>, 256, dyn);
    } else if (threads == 1024) {
        MDG_CUDA(solo_prepare_attr<1024>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<1024>, 1024, dyn);
    } else {
        MDG_CUDA(solo_prepare_attr<512>());
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_solo_persistent<512>, 512, dyn);
    }
    MDG_CUDA(e);
    return MDG_OK;
}

}  // namespace mdg
