// mdg_host.h — host-side objects behind the opaque C-ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "mdg_internal.cuh"

namespace mdg {

void set_error(const std::string& msg);
int cuda_status(cudaError_t e, const char* what);

#define MDG_CUDA(call)                                            \
    do {                                                          \
        cudaError_t e__ = (call);                                 \
        if (e__ != cudaSuccess) return ::mdg::cuda_status(e__, #call); \
    } while (0)

#define MDG_LAUNCHED(ctx)                                            \
    do {                                                             \
        (ctx)->launches++;                                           \
        cudaError_t e__ = cudaGetLastError();                        \
        if (e__ != cudaSuccess) return ::mdg::cuda_status(e__, "kernel launch"); \
    } while (0)

// Fields permuted together at every rebuild.
enum F64Field {
    RX, RY, RZ, VX, VY, VZ, FX, FY, FZ, MASS, RCUT, RNS, EP, EM, NC,
    V0, V1, V2, V3, V4, V5, V6, V7, V8, NF64
};
enum U32Field { ORIG, UID, NU32 };
enum U16Field { KIND, TAG, NU16 };

struct DevArray {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace mdg

struct mdg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t io_stream = nullptr;  // result downloads overlapped with a step (created on first use)
    uint64_t launches = 0;
    int num_sms = 0;
    // lifetime: the caller's handle plus one per live system; the context
    // is freed when both the handle is destroyed and no system remains
    int refs = 1;
    int closed = 0;
    // per-stage event timing (mdg_ctx_set_timing)
    int timing = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending[5];
    double stage_ms[5] = {0, 0, 0, 0, 0};
    uint64_t stage_n[5] = {0, 0, 0, 0, 0};
};

namespace mdg {
enum : int { STALE_EP_V = 1, STALE_EM = 2 };
// Records a start event for `which` when timing is on (else returns null).
cudaEvent_t timer_begin(mdg_ctx* ctx);
void timer_end(mdg_ctx* ctx, int which, cudaEvent_t start);
}  // namespace mdg

// thermostat::Langevin (one term) or thermostat::Compound (parts in order).
struct mdg_thermostat {
    int compound = 0;
    mdg_langevin p{};
    std::vector<mdg_thermostat*> parts;
};

struct mdg_potential {
    int type = 0;  // mdg::POT_LJCUT, POT_EAM or POT_TAB (tabulated Pair: EAM layout, zero rho/F rows)
    double rcut = 0.0;
    // LJsCut
    double a = 0, s = 0, s6 = 0, lj1 = 0, lj2 = 0, factor = 0;
    // LJs (LJs.cxx:7-29)
    double ljs_rVr1 = 0, ljs_rVr2 = 0, ljs_aLJ = 0, ljs_bLJ = 0, ljs_aLJ3 = 0, ljs_bLJ2 = 0, ljs_aVr = 0,
           ljs_aVr2 = 0;
    // EAM host tables (padded by one element) and device copies
    int Nr1 = 0, Nrh1 = 0;
    double dr = 0, drh = 0, dr1 = 0, drh1 = 0;
    std::vector<double> Rho, dRho, Vpar, dVpar, Femb, dFemb;
    int device = -1;
    double* d_tab64 = nullptr;   // Rho,dRho,Vpar,dVpar (Nr1+1 each), Femb,dFemb (Nrh1+1 each)
    float4* d_tab32 = nullptr;   // rho_c, v_c (Nr1 each), f_c (Nrh1)
};

struct mdg_solver {
    int multi = 0;
    int nkinds = 1;
    int periodic = 0;
    int precision = MDG_PREC_FP64;
    int nstages = 0;
    int stages[2] = {0, 0};  // 0 charge, 1 forces
    mdg_potential* pot[mdg::kMaxKinds][mdg::kMaxKinds] = {};
    mdg_thermostat* thermo = nullptr;  // applied after the force stage
};

struct mdg_system {
    mdg_ctx* ctx = nullptr;
    mdg_domain dom{};
    int dim = 3;
    size_t n = 0;
    size_t np = 0;  // n rounded up to 32

    // permuted fields, double-buffered (cur = index of the live buffer)
    int cur = 0;
    double* f64[mdg::NF64][2] = {};
    float* f32[3][2] = {};
    uint32_t* u32[mdg::NU32][2] = {};
    uint16_t* u16[mdg::NU16][2] = {};

    // rebuilt per list build (slot order)
    double* Rc[3] = {};        // cell centres
    uint32_t* cellp = nullptr; // packed local cell coordinates
    int4* pos32 = nullptr;     // fixed-point offsets from the cell centre + w (EAM F' bits); 2 x np
    int4* q0 = nullptr;        // fixed-point offsets at the rebuild (mixed rebuild test)
    float4* o0 = nullptr;      // FP32 offsets at the rebuild (list build prefilter)
    double* r0[3] = {};        // positions at the rebuild (skin test, FP64 form)
    double* saved_rcut = nullptr;
    double* saved_rns = nullptr;
    uint32_t* saved_uid = nullptr;
    uint32_t* slot_of = nullptr;  // caller index -> slot
    uint8_t* bc = nullptr;        // Periodic boundary flag
    double* Fp64 = nullptr;       // F'(nc) per kind column [nk][np] (FP64 form)
    float* Fp32 = nullptr;        // F'(rho) per kind column [nk][np] (mixed Multi)
    float2* trig32 = nullptr;     // (skin/2)^2 per atom (-1: skin <= 0) and its exactness band (mixed rebuild test)
    int force_prec = MDG_PREC_FP64;  // arithmetic of the forces last computed
    int fp_ok = 0;                   // Fp64 = F'(nc) of the current nc (set by the FP64 density pass)
    // Measurement outputs a step's prepare clears (Pair::prepare_one) and
    // this build leaves in place during steps: cleared when next read
    // (STALE_* bits; settle_outputs).
    int stale_out = 0;
    // launch shapes (MDG_SHAPE_*; 0 = the measured default)
    int shape[3] = {0, 0, 0};

    // rebuild scratch
    uint32_t* key = nullptr;
    uint32_t* rank = nullptr;
    uint32_t* src = nullptr;
    uint32_t* bin_count = nullptr;
    uint32_t* bin_start = nullptr;  // nbins + 1
    uint32_t* scan_tmp = nullptr;
    size_t bin_cap = 0;
    size_t scan_cap = 0;  // scan_tmp elements
    double* part = nullptr;  // per-block bounds partials
    size_t part_cap = 0;

    // neighbour list (ELL)
    uint32_t* nbr = nullptr;
    uint32_t* ncnt = nullptr;
    int K = 0;        // capacity per atom (self excluded)
    // the mixed density pass's FP64 cut decisions of the pairs in the band
    // around the cutoff, one bit per list entry (word w of atom i at
    // cutbits[w * np + i], written when the word holds such a pair), for a
    // force pass that starts the next step and so must not read positions it
    // moves; cut_words words per atom, allocated by the step loop that uses
    // them
    uint32_t* cutbits = nullptr;
    int cut_words = 0;
    int half = 0;
    int have_list = 0;
    uint64_t rebuilds = 0;
    int cap_ready = 0;        // bin and list capacities sized
    uint64_t cap_version = 0; // bumped when a capacity buffer is reallocated

    // captured step loop (mdg_run): graph of the driver loop, rebuilt when
    // capacities, the solver, dt or the precision change
    cudaGraphExec_t run_exec = nullptr;
    cudaGraph_t run_graph = nullptr;
    uint64_t run_key[4] = {0, 0, 0, 0};
    unsigned long long* dcounter = nullptr;  // steps left (device)
    unsigned long long* hcounter = nullptr;  // its read-back (pinned)
    long run_launched = 0;                   // steps handed to the last graph launch
    int run_step_kernels = 0;                // kernels per step / per rebuild in the graph
    int run_rebuild_kernels = 0;
    int run_pre_kernels = 0;                 // kernels of the graph's prefix
    double graph_build_s = 0.0;              // host seconds spent building run graphs
    int solo_threads = 0;                    // > 0: run loops as one block of this many threads (solo.cu)

    // device status + grid
    mdg::DevStatus* dstat = nullptr;
    mdg::GridParams* dgrid = nullptr;
    mdg::GridParams grid{};        // host copy of the last rebuild
    mdg::GridParams* hgrid = nullptr;  // pinned
    mdg::DevStatus* hstat = nullptr;   // pinned
    double* red = nullptr;             // reduction scratch (device)
    double* hred = nullptr;            // pinned
    int dirty = 1;                     // host-side changes since the last list

    // pinned staging for host transfers
    void* pin = nullptr;
    size_t pin_bytes = 0;

    // Allocation mode. With a pool, every device buffer of the system comes
    // stream-ordered from it and is released with cudaFreeAsync, so creating
    // and destroying systems never waits for the whole device; the pinned
    // host buffers then belong to the owner (host_borrowed) and the transfer
    // staging is per system (xfer).
    cudaMemPool_t pool = nullptr;
    int host_borrowed = 0;
    void* xfer = nullptr;
    size_t xfer_bytes = 0;
    size_t dev_bytes = 0;  // device bytes held now
    int lazy_init = 0;     // buffers cleared by their first kernel (fused loop), not on the stream
    // one-step host runs: caller-order staging of positions, forces and
    // velocities (3 x n x 3 doubles) and the events that order them
    double* step_io = nullptr;
    size_t step_io_bytes = 0;
    cudaEvent_t step_ev[7] = {};

    double* cur64(int f) { return f64[f][cur]; }
    float* cur32(int c) { return f32[c][cur]; }
    uint32_t* curu32(int f) { return u32[f][cur]; }
    uint16_t* curu16(int f) { return u16[f][cur]; }
};

namespace mdg {
// Device buffers of a system (pool-ordered on its stream when it has a pool).
int sys_malloc(mdg_system* sys, void** p, size_t bytes);
void sys_free(mdg_system* sys, void* p, size_t bytes);
int system_alloc(mdg_system* sys);
void system_free(mdg_system* sys);
// Memory a system is given instead of allocating its own: a device pool and
// the owner's pinned status words and transfer staging.
struct SystemMemory {
    cudaMemPool_t pool = nullptr;
    GridParams* hgrid = nullptr;
    DevStatus* hstat = nullptr;
    double* hred = nullptr;  // 16 doubles
    unsigned long long* hcounter = nullptr;
    void* pin = nullptr;
    size_t pin_bytes = 0;
    int lazy_init = 0;  // leave clearing the buffers to the system's first kernel
};
int system_create(mdg_ctx* ctx, const mdg_domain* domain, size_t n, const SystemMemory* mem, mdg_system** out);
void system_release(mdg_system* sys);
size_t system_base_bytes(size_t n);
// Graph-driven run split for callers that overlap systems: begin checks the
// system, prepares it and launches `steps` steps without waiting; end runs
// once the stream's work is complete and relaunches what an overflowed
// rebuild left (returns 1 when it relaunched, 0 when the run is finished).
int run_async_begin(mdg_solver* s, mdg_system* sys, double dt, long steps);
int run_async_end(mdg_solver* s, mdg_system* sys, double dt, int* relaunched);
int request_begin(mdg_solver* s, mdg_system* sys, const mdg_atom* atoms, double dt, long steps,
                  DevStatus* first_status);
int download_atoms_enqueue(mdg_system* sys, size_t n);
// A solver's potential parameters on the device (valid after a check on a
// system of that device) and, optionally, their host copy.
const PotSet* solver_potsets(mdg_solver* s, PotSet* host);
const ThermoDev* thermo_of(mdg_solver* s);
int settle_outputs(mdg_system* sys);
// Ep and V of atoms with tag != 0 cleared (before an accumulating pass).
int launch_zero_meas(mdg_system* sys);
int nlist_capacity_host(mdg_system* sys, const mdg_atom* atoms, size_t n, int half);
// The fused one-block driver loop (solo.cu): small mixed-precision systems,
// one request per block of a persistent kernel fed through a queue.
constexpr int kSoloRing = 4096;
constexpr int kSoloMaxBlocks = 4096;
// Launches of the persistent kernel that may be in flight at once: a new
// launch tops the kernel up when blocks have exited while others still run
// requests, so its slot must be one whose earlier launch has ended.
constexpr int kSoloGens = 4;
struct SoloQueue {              // host-mapped
    volatile uint32_t tail;     // entries published
    volatile uint32_t stop;     // 1: blocks exit when they find no entry
    uint32_t pad[14];
    int ring[kSoloRing];        // argument-record index of each entry
    // per launch slot and block: 0 exited (or not launched), 1 launched and
    // waiting for an entry (set by the host before the launch, so blocks not
    // yet resident count), 2 running a request
    volatile uint32_t live[kSoloGens][kSoloMaxBlocks];
};
int solo_eligible(const mdg_solver* s, const mdg_system* sys);
size_t solo_args_bytes();
size_t solo_out_bytes();
// Fills the argument record at `args` (host-mapped) of a fresh system's
// whole request: its block clears the system's buffers, loads the atoms from
// atoms_in_dev, builds the first list, computes the initial forces and runs
// `steps` steps; it writes the result atoms to atoms_out_dev and its
// completion record (done = seq) to out_dev (device views of host-mapped
// memory; in and out may be the same buffer).
void solo_fill(void* args, mdg_system* sys, const PotSet* dps, int any_eam, double pot_rcut, int periodic,
               double dt, long steps, const void* atoms_in_dev, void* out_dev, void* atoms_out_dev, uint32_t seq);
int solo_out_read(const void* out_host, uint32_t* done, unsigned long long* left, DevStatus* st,
                  double* service_s = nullptr);
int solo_persistent_launch(cudaStream_t stream, int threads, int blocks, const void* desc_dev, SoloQueue* q_dev,
                           uint32_t* head, int idle_limit, int gen);
int solo_blocks_per_sm(int threads, int* blocks);
// The persistent kernel inside a captured graph: one executable graph per
// launch slot, made by capturing that slot's first launch on its stream;
// a later launch sets the graph's kernel node to the blocks it wants and
// launches the graph again.
struct SoloGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t node = nullptr;
};
int solo_graph_launch(SoloGraph& G, cudaStream_t stream, int threads, int blocks, const void* desc_dev,
                      SoloQueue* q_dev, uint32_t* head, int idle_limit, int gen);
void solo_graph_destroy(SoloGraph& G);
int nlist_build(mdg_system* sys, double kbuf, int half);
int nlist_sort_perm(mdg_system* sys, uint32_t* perm);
int pot_eval(const PotParams& P, int what, const double* x, size_t n, double* out0, double* out1,
             cudaStream_t st);
int nlist_list_for(mdg_system* sys, const double x[3], std::vector<uint64_t>& found);
// One atom's force / virial / density over an explicit list (forces.cu):
// recs_host[0] is the atom, slots_host[k] the record of list entry k; the
// records come back updated. Waits on `st`.
int pot_atom(const PotParams& P, int what, mdg_atom* recs_host, size_t nrec, const uint32_t* slots_host,
             size_t count, int half, cudaStream_t st, uint32_t* flags);
// Grid::build alone (nlist.cu): the bounds pass and the grid over the
// system's atoms, waited for.
int grid_build_only(mdg_system* sys, GridParams* out);
int nlist_export_offsets(mdg_system* sys, std::vector<uint64_t>& off);
int nlist_export_entries(mdg_system* sys, const std::vector<uint64_t>& off, uint64_t* idx);
int nlist_capacity(mdg_system* sys, int half);
int nlist_enqueue(mdg_system* sys);
int potset_build(mdg_solver* s, mdg_system* sys, PotSet* out);
int pot_upload(mdg_potential* p, int device);
int run_prepare(mdg_solver* s, mdg_system* sys, const PotSet& ps, int check_rcut);
int run_stage(mdg_solver* s, mdg_system* sys, const PotSet& ps, int stage);
int run_virials(mdg_solver* s, mdg_system* sys, const PotSet& ps);
int run_drift(mdg_solver* s, mdg_system* sys, const PotSet& ps, double dt);
int run_kick(mdg_solver* s, mdg_system* sys, double dt);
int run_decide(mdg_system* sys);
int ensure_pinned(mdg_system* sys, size_t bytes);
}  // namespace mdg
