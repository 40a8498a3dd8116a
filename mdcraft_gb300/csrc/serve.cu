// serve.cu — continuous batching of independent MD systems on one GPU.
//
// The reference runs one system per process, its driver loop on the host
// (test/python/solver/test-EAM.py:101-200); there is no serving layer to
// mirror. Here a request is a whole driver loop (update(-1), prepare,
// stages, then `steps` x {make_step; if decide(): update(-1)}) over its own
// atoms. Requests wait in a FIFO; each takes a slot when one is free and its
// device footprint fits in the budget left by the running ones. Two ways to
// run a request:
//
// Block mode (mixed precision, one kind, up to 65536 atoms): the request's
// whole run, set-up included, is one thread block of a persistent kernel
// (solo.cu). The host allocates the system's buffers (stream-ordered, from
// the server's pool), sizes its capacities from the atoms and fills the
// block's argument record in host-mapped memory; once the allocations have
// passed it publishes the record in a queue. Blocks of the persistent kernel
// claim queue entries as they finish their previous request, so requests
// that arrive while others run start as soon as a block is free. Each
// block writes its result atoms and a completion record into host-mapped
// memory; the host polls those and never waits for the device. Idle blocks
// exit after a bounded wait; the host tops the kernel up with a further
// launch (up to kSoloGens in flight) whenever fewer blocks are alive than
// the GPU holds and requests wait. Each launch slot's kernel is captured
// once into a CUDA graph; a top-up sets that graph's grid to the blocks
// missing and launches it.
//
// Graph mode (everything else, or when block mode is off): the request's
// system gets the slot's own stream; set-up and the loop (one graph launch)
// are enqueued there, completion is an event, and the result comes back by
// an asynchronous copy.
//
// Results are independent of the mix: every block or kernel reads and
// writes only its own system's buffers, sums in a fixed order and uses no
// atomics across systems, so a request gives the same bits alone or among
// others, in either mode.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mdg_host.h"

using namespace mdg;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    mdg_solver* solver = nullptr;
    mdg_domain dom{};
    std::vector<mdg_atom> atoms;  // input, replaced by the result
    double dt = 0.0;
    long steps = 0;
    int precision = MDG_PREC_FP64;
    size_t footprint = 0;  // bytes charged while it runs
    mdg_request_info info{};
    double t_graph_start = 0.0;  // server clock at the latest admission to a graph loop
};

// A request's work for the admission order: atoms x steps.
inline double work_of(const Request* r) { return (double)r->atoms.size() * (double)r->steps; }

// IDLE -> ALLOC (buffers requested) -> BLOCK (queued or running in a block)
// -> finished, or IDLE -> RUN (graph loop enqueued) -> COPY (result copy
// enqueued) -> finished.
enum SlotState { IDLE = 0, RUN = 1, COPY = 2, BLOCK = 3, ALLOC = 4 };

struct Slot {
    mdg_ctx* ctx = nullptr;  // the slot's own stream (graph mode), made on first use
    cudaEvent_t ev = nullptr;
    Request* req = nullptr;
    mdg_system* sys = nullptr;
    SystemMemory mem;
    int state = IDLE;
    int checked = 0;                    // request set up on the synchronous, checked path
    DevStatus* first_status = nullptr;  // device status after the first list build (pinned)
    void* hblock = nullptr;             // pinned status words of the slot's systems
    void* pin = nullptr;                // host-mapped staging: input atoms, then results
    void* pin_dev = nullptr;            // its device view
    uint32_t seq = 0;                   // completion value of the slot's last block
};

// Slots whose buffers were requested in one pass, published together once
// the allocation stream has passed `ev`.
struct AllocGroup {
    cudaEvent_t ev = nullptr;
    std::vector<int> slots;
};

// Neighbour entries per atom the admission estimate assumes when the atoms
// give no better figure: a dense liquid or solid at rns = rc + skin.
constexpr int kDefaultNeighbours = 96;

// Executable graphs of finished requests held before they are destroyed.
constexpr size_t kMaxSpentGraphs = 16384;

// Polls (about a microsecond apart) after which an idle block of the
// persistent kernel exits.
constexpr int kIdlePolls = 100000;

}  // namespace

struct mdg_server {
    int device = 0;
    cudaMemPool_t pool = nullptr;
    size_t budget = 0, used = 0, peak = 0;
    size_t max_atoms = 0;
    int block_threads = 0;
    int order = MDG_ORDER_FIFO;
    std::vector<Slot> slots;
    mdg_ctx* alloc_ctx = nullptr;  // block-mode systems: allocations and releases
    mdg_ctx* feed_ctx[kSoloGens] = {};     // the persistent kernel: one stream per launch slot
    cudaEvent_t feed_ev[kSoloGens] = {};   // recorded after each launch
    SoloGraph feed_graph[kSoloGens];       // the kernel captured once per launch slot
    int feed_launched[kSoloGens] = {};
    int threads = 512, blocks = 0; // persistent kernel shape
    SoloQueue* q = nullptr;        // host-mapped request queue
    SoloQueue* q_dev = nullptr;
    uint32_t* head = nullptr;      // next entry to claim (device)
    uint32_t published = 0;
    std::deque<AllocGroup> alloc_groups;
    std::vector<cudaEvent_t> free_events;
    std::deque<Request*> queue;
    double queued_work = 0;        // atom-steps of the requests in `queue`
    std::unordered_map<uint64_t, Request*> reqs;
    std::deque<uint64_t> finished;
    uint64_t next_id = 1;
    uint64_t admitted = 0;
    size_t nfinished = 0;
    void* desc = nullptr;       // host-mapped argument records, one per slot
    void* desc_dev = nullptr;
    void* outs = nullptr;       // host-mapped completion records, one per slot
    void* outs_dev = nullptr;
    size_t desc_stride = 0, out_stride = 0;
    uint64_t kernel_launches = 0;
    double admit_s = 0.0, graph_s = 0.0, retire_s = 0.0;
    uint64_t rechecked = 0;
    double graph_destroy_s = 0.0, release_s = 0.0, end_s = 0.0, download_s = 0.0;
    std::vector<cudaGraphExec_t> spent_execs;
    std::vector<cudaGraph_t> spent_graphs;
    Clock::time_point t0;
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes charged for a request: the system's per-atom buffers, the
// list (ELL, K rounded up to 4, at the capacity estimate's margin), the bin
// arrays and the transfer staging.
size_t footprint_of(size_t n, int neighbours) {
    size_t np = (n + 31) & ~size_t(31);
    size_t K = ((size_t)std::max(neighbours, 4) * 135 / 100 + 16 + 3) & ~size_t(3);
    size_t list = K * np * sizeof(uint32_t);
    size_t bins = 2 * (np + 4096) * sizeof(uint32_t) + 64 * 1024;
    size_t xfer = n * sizeof(mdg_atom);
    return system_base_bytes(n) + list + bins + xfer;
}

// Listed neighbours per atom expected from the atoms' number density and
// their largest list radius (the estimate nlist_capacity makes on the
// device, here on the host before anything is allocated).
int neighbours_of(const mdg_domain& d, const mdg_atom* a, size_t n) {
    double rns = 0.0;
    for (size_t i = 0; i < n; ++i) rns = std::max(rns, a[i].rns);
    double vol = 1.0;
    int dim = 0;
    for (int k = 0; k < 3; ++k) {
        double L = d.bmax[k] - d.bmin[k];
        if (L > 1e-15) {
            vol *= L;
            ++dim;
        }
    }
    if (dim == 0 || rns <= 0.0 || n == 0) return kDefaultNeighbours;
    double rho = (double)n / vol;
    double ball = dim == 3 ? 4.18879020478639 * rns * rns * rns : dim == 2 ? 3.14159265358979 * rns * rns : 2.0 * rns;
    double k = rho * ball;
    if (!(k < 1e6)) return kDefaultNeighbours;
    return (int)std::min<double>(std::ceil(k) + 1.0, (double)n);
}

size_t running_of(const mdg_server* sv) {
    size_t k = 0;
    for (const Slot& sl : sv->slots) k += sl.req ? 1 : 0;
    return k;
}

void destroy_spent(mdg_server* sv) {
    double t = sv->now();
    for (cudaGraphExec_t e : sv->spent_execs) cudaGraphExecDestroy(e);
    for (cudaGraph_t g : sv->spent_graphs) cudaGraphDestroy(g);
    sv->spent_execs.clear();
    sv->spent_graphs.clear();
    sv->graph_destroy_s += sv->now() - t;
}

void finish(mdg_server* sv, Request* r, int status) {
    r->info.status = status;
    r->info.done = 1;
    r->info.t_done = sv->now();
    // graph mode: from admission to completion (host clock); a repeat on the
    // checked path adds its own span
    if (r->t_graph_start > 0.0) r->info.service_s += r->info.t_done - r->t_graph_start;
    sv->finished.push_back(r->id);
    sv->nfinished++;
}

// Releases the slot's system (stream-ordered behind its last work) and the
// request's charge.
void retire(mdg_server* sv, Slot& sl) {
    if (sl.sys) {
        sv->graph_s += sl.sys->graph_build_s;
        double t = sv->now();
        // destroying an executable graph waits for the whole device: keep
        // them until no request runs (or the server goes)
        if (sl.sys->run_exec) sv->spent_execs.push_back(sl.sys->run_exec);
        if (sl.sys->run_graph) sv->spent_graphs.push_back(sl.sys->run_graph);
        sl.sys->run_exec = nullptr;
        sl.sys->run_graph = nullptr;
        double t1 = sv->now();
        sv->graph_destroy_s += t1 - t;
        system_release(sl.sys);
        sv->release_s += sv->now() - t1;
        sl.sys = nullptr;
    }
    if (sl.req) {
        sv->used -= std::min(sv->used, sl.req->footprint);
        sl.req = nullptr;
    }
    sl.state = IDLE;
}

void fail(mdg_server* sv, Slot& sl, int rc) {
    Request* r = sl.req;
    r->info.footprint = r->footprint;
    retire(sv, sl);
    finish(sv, r, rc);
}

bool block_mode(const mdg_server* sv, const Request* r) {
    if (sv->block_threads < 0) return false;
    const mdg_solver* s = r->solver;
    return r->precision == MDG_PREC_MIXED && !s->multi && s->nstages >= 1 && r->atoms.size() <= 65536 &&
           r->atoms.size() > 0;
}

void charge(mdg_server* sv, Slot& sl, Request* r) {
    sl.req = r;
    r->info.t_admit = sv->now();
    sv->admitted++;
    sv->used += r->footprint;
    sv->peak = std::max(sv->peak, sv->used);
}

void charge_actual(mdg_server* sv, Slot& sl, Request* r) {
    // charge what the system holds once its capacities are sized
    if (sl.sys && sl.sys->dev_bytes > r->footprint) {
        sv->used += sl.sys->dev_bytes - r->footprint;
        r->footprint = sl.sys->dev_bytes;
        sv->peak = std::max(sv->peak, sv->used);
    }
}

int ensure_slot_ctx(mdg_server* sv, Slot& sl) {
    if (sl.ctx) return MDG_OK;
    int rc = mdg_ctx_create(sv->device, &sl.ctx);
    if (rc) return rc;
    MDG_CUDA(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
    return MDG_OK;
}

// Graph mode: set-up and loop enqueued on the slot's stream (checked = the
// driver's calls one by one, each list build verified and grown).
void admit_graph(mdg_server* sv, Slot& sl, Request* r, int checked) {
    double t0 = sv->now();
    r->t_graph_start = t0;
    sl.checked = checked;
    size_t n = r->atoms.size();
    int rc = ensure_slot_ctx(sv, sl);
    if (rc == MDG_OK) rc = system_create(sl.ctx, &r->dom, n, &sl.mem, &sl.sys);
    int prec_saved = r->solver->precision;
    r->solver->precision = r->precision;
    if (rc == MDG_OK && !checked) {
        rc = request_begin(r->solver, sl.sys, r->atoms.data(), r->dt, r->steps, sl.first_status);
    } else if (rc == MDG_OK) {
        rc = mdg_system_upload_atoms(sl.sys, r->atoms.data(), n);
        if (rc == MDG_OK) {
            rc = mdg_nlist_update(sl.sys, -1.0, 0);
            if (rc == MDG_ERR_RANGE) rc = MDG_OK;  // flagged in the system's status, as in mdg_run
        }
        if (rc == MDG_OK) rc = mdg_solver_prepare(r->solver, sl.sys);
        if (rc == MDG_OK) rc = mdg_solver_stages(r->solver, sl.sys);
        if (rc == MDG_OK) rc = run_async_begin(r->solver, sl.sys, r->dt, r->steps);
    }
    r->solver->precision = prec_saved;
    if (rc == MDG_OK) {
        charge_actual(sv, sl, r);
        cudaError_t e = cudaEventRecord(sl.ev, sl.ctx->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "slot event");
    }
    sv->admit_s += sv->now() - t0;
    if (rc != MDG_OK) {
        fail(sv, sl, rc);
        return;
    }
    sl.state = RUN;
}

// Block mode: the system's buffers requested on the allocation stream and
// its argument record filled; published once the allocations have passed.
bool admit_block(mdg_server* sv, Slot& sl, Request* r) {
    double t0 = sv->now();
    size_t k = &sl - sv->slots.data();
    size_t n = r->atoms.size();
    SystemMemory mem = sl.mem;
    mem.lazy_init = 1;
    int rc = system_create(sv->alloc_ctx, &r->dom, n, &mem, &sl.sys);
    PotSet ps;
    int prec_saved = r->solver->precision;
    r->solver->precision = r->precision;
    if (rc == MDG_OK) {
        memcpy(sl.pin, r->atoms.data(), n * sizeof(mdg_atom));
        rc = nlist_capacity_host(sl.sys, r->atoms.data(), n, 0);
    }
    if (rc == MDG_OK) {
        sl.sys->grid = *sl.sys->hgrid;
        rc = potset_build(r->solver, sl.sys, &ps);
    }
    if (rc == MDG_OK) {
        const mdg_solver* s = r->solver;
        double pot_rcut = s->multi ? -1.0 : s->pot[0][0]->rcut;
        sl.seq++;
        solo_fill((char*)sv->desc + k * sv->desc_stride, sl.sys, solver_potsets(r->solver, nullptr), ps.any_eam,
                  pot_rcut, s->periodic, r->dt, r->steps, sl.pin_dev, (char*)sv->outs_dev + k * sv->out_stride,
                  sl.pin_dev, sl.seq);
        sl.sys->have_list = 1;
        sl.sys->dirty = 0;
        sl.sys->rebuilds = 1;
        sl.sys->force_prec = MDG_PREC_MIXED;
        charge_actual(sv, sl, r);
    }
    r->solver->precision = prec_saved;
    sv->admit_s += sv->now() - t0;
    if (rc != MDG_OK) {
        fail(sv, sl, rc);
        return false;
    }
    sl.state = ALLOC;
    sl.checked = 0;
    return true;
}

// Graph mode: the slot's event has passed; advance its request one state.
void advance_graph(mdg_server* sv, Slot& sl) {
    double t = sv->now();
    Request* r = sl.req;
    if (sl.state == RUN) {
        if (!sl.checked && (sl.first_status->build_flags & FLAG_OVERFLOW)) {
            // the first list outgrew the capacities sized on the host: the
            // run is void; repeat it on the checked path
            if (sl.sys) {
                sv->graph_s += sl.sys->graph_build_s;
                system_release(sl.sys);
                sl.sys = nullptr;
            }
            sv->rechecked++;
            sv->retire_s += sv->now() - t;
            admit_graph(sv, sl, r, 1);
            return;
        }
        int prec_saved = r->solver->precision;
        r->solver->precision = r->precision;
        int relaunched = 0;
        double t0 = sv->now();
        int rc = run_async_end(r->solver, sl.sys, r->dt, &relaunched);
        r->solver->precision = prec_saved;
        double t1 = sv->now();
        sv->end_s += t1 - t0;
        if (rc == MDG_OK && !relaunched) rc = download_atoms_enqueue(sl.sys, r->atoms.size());
        sv->download_s += sv->now() - t1;
        if (rc == MDG_OK) {
            cudaError_t e = cudaEventRecord(sl.ev, sl.ctx->stream);
            if (e != cudaSuccess) rc = cuda_status(e, "slot event");
        }
        if (rc != MDG_OK) {
            fail(sv, sl, rc);
        } else if (!relaunched) {
            sl.state = COPY;
        }
        sv->retire_s += sv->now() - t;
        return;
    }
    // COPY: the result is in the slot's pinned staging
    memcpy(r->atoms.data(), sl.pin, r->atoms.size() * sizeof(mdg_atom));
    r->info.rebuilds = sl.sys->rebuilds;
    r->info.footprint = r->footprint;
    retire(sv, sl);
    finish(sv, r, MDG_OK);
    sv->retire_s += sv->now() - t;
}

// Block mode: the slot's block has written its completion record.
void advance_block(mdg_server* sv, Slot& sl, unsigned long long left, const DevStatus& st) {
    double t = sv->now();
    Request* r = sl.req;
    if (st.pad[1] != 0 || left != 0) {
        // a list outgrew the capacities sized on the host: the run is void;
        // repeat it on the checked path (graph mode, capacities grown there)
        if (sl.sys) {
            system_release(sl.sys);
            sl.sys = nullptr;
        }
        sv->rechecked++;
        sv->retire_s += sv->now() - t;
        admit_graph(sv, sl, r, 1);
        return;
    }
    memcpy(r->atoms.data(), sl.pin, r->atoms.size() * sizeof(mdg_atom));
    sl.sys->rebuilds += st.pad[0];
    r->info.rebuilds = sl.sys->rebuilds;
    r->info.footprint = r->footprint;
    retire(sv, sl);
    finish(sv, r, MDG_OK);
    sv->retire_s += sv->now() - t;
}

int progress(mdg_server* sv) {
    MDG_CUDA(cudaSetDevice(sv->device));
    for (size_t k = 0; k < sv->slots.size(); ++k) {
        Slot& sl = sv->slots[k];
        if (!sl.req || sl.state == ALLOC) continue;
        if (sl.state == BLOCK) {
            uint32_t done = 0;
            unsigned long long left = 0;
            DevStatus st;
            double service = 0.0;
            solo_out_read((char*)sv->outs + k * sv->out_stride, &done, &left, &st, &service);
            if (done == sl.seq) {
                sl.req->info.service_s += service;
                advance_block(sv, sl, left, st);
            }
            continue;
        }
        cudaError_t e = cudaEventQuery(sl.ev);
        if (e == cudaErrorNotReady) continue;
        if (e != cudaSuccess) {
            fail(sv, sl, cuda_status(e, "request"));
            continue;
        }
        advance_graph(sv, sl);
    }
    // publish the records whose allocations have passed
    while (!sv->alloc_groups.empty()) {
        AllocGroup& ag = sv->alloc_groups.front();
        cudaError_t e = cudaEventQuery(ag.ev);
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess) return cuda_status(e, "allocation event");
        for (int k : ag.slots) {
            Slot& sl = sv->slots[k];
            if (sl.state != ALLOC) continue;
            sv->q->ring[sv->published % kSoloRing] = k;
            sv->published++;
            sl.state = BLOCK;
        }
        std::atomic_thread_fence(std::memory_order_seq_cst);  // records and ring before the tail
        sv->q->tail = sv->published;
        sv->free_events.push_back(ag.ev);
        sv->alloc_groups.pop_front();
    }
    // spent graphs go when the device is idle (or too many are held)
    if (!sv->spent_execs.empty() &&
        ((sv->queue.empty() && running_of(sv) == 0) || sv->spent_execs.size() >= kMaxSpentGraphs))
        destroy_spent(sv);
    // Admission in FIFO order; with MDG_ORDER_LARGEST the largest waiting
    // request first; with MDG_ORDER_BALANCED the largest first only while
    // its atom-steps are at least the waiting atom-steps per worker (the
    // persistent kernel's blocks, or the request slots without it): once
    // the backlog is short enough that it would otherwise run on alone at
    // the end (longest-first on the tail, the rule that bounds a schedule's
    // makespan). The chosen request waits for memory rather than being
    // overtaken.
    AllocGroup group;
    for (Slot& sl : sv->slots) {
        if (sv->queue.empty()) break;
        if (sl.req) continue;
        auto pick = sv->queue.begin();
        if (sv->order != MDG_ORDER_FIFO) {
            auto largest = sv->queue.begin();
            for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it)
                if (work_of(*it) > work_of(*largest)) largest = it;
            const double per = sv->block_threads >= 0 ? (double)sv->blocks : (double)sv->slots.size();
            if (sv->order == MDG_ORDER_LARGEST || work_of(*largest) * per >= sv->queued_work) pick = largest;
        }
        Request* r = *pick;
        if (sv->used + r->footprint > sv->budget && sv->used > 0) break;
        sv->queue.erase(pick);
        sv->queued_work = sv->queue.empty() ? 0.0 : sv->queued_work - work_of(r);
        charge(sv, sl, r);
        if (!block_mode(sv, r)) {
            admit_graph(sv, sl, r, 0);
            continue;
        }
        if (admit_block(sv, sl, r)) group.slots.push_back((int)(&sl - sv->slots.data()));
    }
    if (!group.slots.empty()) {
        if (sv->free_events.empty()) {
            cudaEvent_t ev;
            MDG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            sv->free_events.push_back(ev);
        }
        group.ev = sv->free_events.back();
        sv->free_events.pop_back();
        MDG_CUDA(cudaEventRecord(group.ev, sv->alloc_ctx->stream));
        sv->alloc_groups.push_back(std::move(group));
    }
    // the persistent kernel: topped up when requests wait and fewer of its
    // blocks are alive (running a request, waiting for one, or launched and
    // not yet resident) than the smaller of the blocks the GPU holds and the
    // requests published. Idle blocks exit after a bounded wait, so blocks of
    // one launch can be gone while others of it still run long requests; a
    // top-up launches the missing blocks in a launch slot whose previous
    // launch has ended, with their flags set before the launch so that
    // blocks not yet resident are counted.
    size_t waiting = 0;
    for (const Slot& sl : sv->slots) waiting += (sl.req && sl.state == BLOCK) ? 1 : 0;
    if (waiting > 0) {
        int alive = 0, free_gen = -1;
        for (int gen = 0; gen < kSoloGens; ++gen) {
            bool ended = true;
            if (sv->feed_launched[gen]) {
                cudaError_t e = cudaEventQuery(sv->feed_ev[gen]);
                if (e == cudaErrorNotReady) ended = false;
                else if (e != cudaSuccess) return cuda_status(e, "persistent kernel");
            }
            if (ended) {
                if (free_gen < 0) free_gen = gen;
                continue;
            }
            for (int b = 0; b < sv->blocks; ++b) alive += sv->q->live[gen][b] ? 1 : 0;
        }
        if ((size_t)alive < std::min<size_t>((size_t)sv->blocks, waiting) && free_gen >= 0) {
            const int k = sv->blocks - alive;
            // an ended launch left every flag of its slot at 0
            for (int b = 0; b < k; ++b) sv->q->live[free_gen][b] = 1u;
            std::atomic_thread_fence(std::memory_order_seq_cst);
            int rc = solo_graph_launch(sv->feed_graph[free_gen], sv->feed_ctx[free_gen]->stream, sv->threads, k,
                                       sv->desc_dev, sv->q_dev, sv->head, kIdlePolls, free_gen);
            if (rc) {
                for (int b = 0; b < k; ++b) sv->q->live[free_gen][b] = 0u;
                return rc;
            }
            MDG_CUDA(cudaEventRecord(sv->feed_ev[free_gen], sv->feed_ctx[free_gen]->stream));
            sv->feed_launched[free_gen] = 1;
            sv->kernel_launches++;
        }
    }
    return MDG_OK;
}

void server_free(mdg_server* sv) {
    cudaSetDevice(sv->device);
    if (sv->q) sv->q->stop = 1;
    for (mdg_ctx* c : sv->feed_ctx)
        if (c) cudaStreamSynchronize(c->stream);
    if (sv->alloc_ctx) cudaStreamSynchronize(sv->alloc_ctx->stream);
    for (Slot& sl : sv->slots) {
        if (sl.ctx) cudaStreamSynchronize(sl.ctx->stream);
        if (sl.sys) retire(sv, sl);
    }
    if (sv->alloc_ctx) cudaStreamSynchronize(sv->alloc_ctx->stream);
    for (Slot& sl : sv->slots) {
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.hblock) cudaFreeHost(sl.hblock);
        if (sl.pin) cudaFreeHost(sl.pin);
        if (sl.ctx) mdg_ctx_destroy(sl.ctx);
    }
    for (AllocGroup& ag : sv->alloc_groups) sv->free_events.push_back(ag.ev);
    for (cudaEvent_t e : sv->free_events) cudaEventDestroy(e);
    for (int g = 0; g < kSoloGens; ++g) {
        solo_graph_destroy(sv->feed_graph[g]);
        if (sv->feed_ev[g]) cudaEventDestroy(sv->feed_ev[g]);
        if (sv->feed_ctx[g]) mdg_ctx_destroy(sv->feed_ctx[g]);
    }
    if (sv->alloc_ctx) mdg_ctx_destroy(sv->alloc_ctx);
    destroy_spent(sv);
    for (auto& kv : sv->reqs) delete kv.second;
    if (sv->desc) cudaFreeHost(sv->desc);
    if (sv->outs) cudaFreeHost(sv->outs);
    if (sv->q) cudaFreeHost(sv->q);
    if (sv->head) cudaFree(sv->head);
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    delete sv;
}

}  // namespace

extern "C" {

size_t mdg_server_footprint(size_t n, int neighbours) { return footprint_of(n, neighbours); }

int mdg_server_create(int device, const mdg_server_config* cfg, mdg_server** out) {
    if (!cfg || !out || cfg->slots < 1 || cfg->slots > kSoloRing || cfg->max_atoms == 0 || cfg->max_atoms >= kMaxAtoms)
        return MDG_ERR_INVALID;
    if (cfg->block_threads > 0 && cfg->block_threads != 256 && cfg->block_threads != 512 &&
        cfg->block_threads != 640 && cfg->block_threads != 768 && cfg->block_threads != 896 &&
        cfg->block_threads != 1024)
        return MDG_ERR_INVALID;
    if (cfg->order != MDG_ORDER_FIFO && cfg->order != MDG_ORDER_LARGEST && cfg->order != MDG_ORDER_BALANCED)
        return MDG_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error("no CUDA device available (libmdg has no CPU fallback)");
        return MDG_ERR_NODEV;
    }
    if (device < 0 || device >= count) return MDG_ERR_INVALID;
    MDG_CUDA(cudaSetDevice(device));
    mdg_server* sv = new mdg_server();
    sv->device = device;
    sv->t0 = Clock::now();
    sv->max_atoms = cfg->max_atoms;
    sv->block_threads = cfg->block_threads;
    sv->order = cfg->order;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) {
        server_free(sv);
        return cuda_status(e, "cudaMemGetInfo");
    }
    sv->budget = cfg->hbm_budget ? cfg->hbm_budget : free_b / 2;

    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    e = cudaMemPoolCreate(&sv->pool, &props);
    if (e == cudaSuccess) {
        // keep released memory in the pool: retiring a request must not
        // hand pages back to the driver and admitting the next map them again
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) {
        // memory freed on one stream is not handed to another stream before
        // the free has completed (no dependency between streams)
        int no = 0;
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    const size_t nslots = (size_t)cfg->slots;
    if (e == cudaSuccess) {
        sv->desc_stride = solo_args_bytes();  // the launch indexes the records as an array
        sv->out_stride = (solo_out_bytes() + 255) & ~size_t(255);
        e = cudaHostAlloc(&sv->desc, nslots * sv->desc_stride, cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&sv->desc_dev, sv->desc, 0);
        if (e == cudaSuccess) e = cudaHostAlloc(&sv->outs, nslots * sv->out_stride, cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&sv->outs_dev, sv->outs, 0);
        if (e == cudaSuccess) memset(sv->outs, 0, nslots * sv->out_stride);
    }
    if (e != cudaSuccess) {
        int rc = cuda_status(e, "server memory");
        server_free(sv);
        return rc;
    }
    {
        int rc = mdg_ctx_create(device, &sv->alloc_ctx);
        for (int g = 0; g < kSoloGens && rc == MDG_OK; ++g) rc = mdg_ctx_create(device, &sv->feed_ctx[g]);
        if (rc == MDG_OK) {
            e = cudaSuccess;
            for (int g = 0; g < kSoloGens && e == cudaSuccess; ++g)
                e = cudaEventCreateWithFlags(&sv->feed_ev[g], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaHostAlloc((void**)&sv->q, sizeof(SoloQueue), cudaHostAllocMapped);
            if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&sv->q_dev, sv->q, 0);
            if (e == cudaSuccess) memset((void*)sv->q, 0, sizeof(SoloQueue));
            if (e == cudaSuccess) e = cudaMalloc(&sv->head, sizeof(uint32_t));
            if (e == cudaSuccess) e = cudaMemset(sv->head, 0, sizeof(uint32_t));
            if (e != cudaSuccess) rc = cuda_status(e, "server queue");
        }
        // persistent kernel: block size, and as many blocks as fit on the GPU
        // 768 threads (one block per SM, 80 registers) measured fastest on the
        // serving mix: 2.04-2.08e9 atom-steps/s against 2.06e9 with 896,
        // 2.00e9 with 640, 1.84e9 with 1024 (64 registers, twice the spills)
        sv->threads = cfg->block_threads > 0 ? cfg->block_threads : 768;
        int per_sm = 0;
        if (rc == MDG_OK) rc = solo_blocks_per_sm(sv->threads, &per_sm);
        if (rc != MDG_OK) {
            server_free(sv);
            return rc;
        }
        sv->blocks = std::min(kSoloMaxBlocks, std::max(1, per_sm) * std::max(1, sv->alloc_ctx->num_sms));
    }
    sv->slots.resize(nslots);
    for (Slot& sl : sv->slots) {
        e = cudaMallocHost(&sl.hblock, 1024);
        if (e == cudaSuccess) e = cudaHostAlloc(&sl.pin, cfg->max_atoms * sizeof(mdg_atom), cudaHostAllocMapped);
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&sl.pin_dev, sl.pin, 0);
        if (e != cudaSuccess) {
            int rc = cuda_status(e, "slot");
            server_free(sv);
            return rc;
        }
        char* hb = (char*)sl.hblock;
        sl.mem.pool = sv->pool;
        sl.mem.hgrid = (GridParams*)hb;
        sl.mem.hstat = (DevStatus*)(hb + 512);
        sl.mem.hred = (double*)(hb + 640);
        sl.mem.hcounter = (unsigned long long*)(hb + 768);
        sl.first_status = (DevStatus*)(hb + 896);
        sl.mem.pin = sl.pin;
        sl.mem.pin_bytes = cfg->max_atoms * sizeof(mdg_atom);
        static_assert(sizeof(GridParams) <= 512 && sizeof(DevStatus) <= 128, "slot host block layout");
    }
    *out = sv;
    return MDG_OK;
}

int mdg_server_destroy(mdg_server* srv) {
    if (!srv) return MDG_ERR_INVALID;
    server_free(srv);
    return MDG_OK;
}

int mdg_server_submit(mdg_server* srv, mdg_solver* solver, const mdg_domain* domain, const mdg_atom* atoms,
                      size_t n, double dt, long steps, uint64_t* id) {
    if (!srv || !solver || !domain || (!atoms && n) || !id || steps < 0) return MDG_ERR_INVALID;
    if (n > srv->max_atoms) {
        set_error("request larger than the server's max_atoms");
        return MDG_ERR_INVALID;
    }
    if (solver->precision == MDG_PREC_MIXED && solver->periodic && n) {
        // as the mixed stages require: every periodic box edge at least 2 rns
        double mr = 0.0;
        for (size_t k = 0; k < n; ++k) mr = std::max(mr, atoms[k].rns);
        for (int a = 0; a < 3; ++a) {
            const double L = domain->bmax[a] - domain->bmin[a];
            if (domain->periodic[a] && L > 0.0 && L < 2.0 * mr) {
                set_error("the mixed form needs every periodic box edge to be at least 2 rns; use an FP64 solver "
                          "for this request");
                return MDG_ERR_INVALID;
            }
        }
    }
    size_t fp = footprint_of(n, neighbours_of(*domain, atoms, n));
    if (fp > srv->budget) {
        set_error("request footprint exceeds the server's device-memory budget");
        return MDG_ERR_NOMEM;
    }
    Request* r = new Request();
    r->id = srv->next_id++;
    r->solver = solver;
    r->dom = *domain;
    r->atoms.assign(atoms, atoms + n);
    r->dt = dt;
    r->steps = steps;
    r->precision = solver->precision;
    r->footprint = fp;
    r->info.t_submit = srv->now();
    srv->reqs[r->id] = r;
    *id = r->id;
    if (n == 0 || steps == 0) {
        // nothing to run: the input is the result
        finish(srv, r, MDG_OK);
        return MDG_OK;
    }
    srv->queue.push_back(r);
    srv->queued_work += work_of(r);
    return MDG_OK;
}

int mdg_server_progress(mdg_server* srv, size_t* running) {
    if (!srv) return MDG_ERR_INVALID;
    int rc = progress(srv);
    if (running) *running = running_of(srv);
    return rc;
}

int mdg_server_poll(mdg_server* srv, uint64_t* ids, size_t cap, size_t* count) {
    if (!srv || (!ids && cap) || !count) return MDG_ERR_INVALID;
    int rc = progress(srv);
    size_t k = 0;
    while (k < cap && !srv->finished.empty()) {
        ids[k++] = srv->finished.front();
        srv->finished.pop_front();
    }
    *count = k;
    return rc;
}

int mdg_server_wait(mdg_server* srv, uint64_t id, double timeout_s) {
    if (!srv) return MDG_ERR_INVALID;
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return MDG_ERR_INVALID;
    Request* r = it->second;
    double t_end = srv->now() + timeout_s;
    while (!r->info.done) {
        int rc = progress(srv);
        if (rc) return rc;
        if (r->info.done) break;
        if (srv->now() > t_end) return MDG_ERR_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return MDG_OK;
}

int mdg_server_result(mdg_server* srv, uint64_t id, mdg_atom* atoms, size_t n, mdg_request_info* info) {
    if (!srv) return MDG_ERR_INVALID;
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return MDG_ERR_INVALID;
    Request* r = it->second;
    if (!r->info.done) return MDG_ERR_STATE;
    if (atoms && n != r->atoms.size()) return MDG_ERR_INVALID;
    if (atoms) memcpy(atoms, r->atoms.data(), n * sizeof(mdg_atom));
    if (info) *info = r->info;
    // an id handed out by poll but not yet read stays in `finished` only
    // until polled; drop it there too
    auto f = std::find(srv->finished.begin(), srv->finished.end(), id);
    if (f != srv->finished.end()) srv->finished.erase(f);
    srv->reqs.erase(it);
    delete r;
    return MDG_OK;
}

int mdg_server_stats_get(mdg_server* srv, mdg_server_stats* out) {
    if (!srv || !out) return MDG_ERR_INVALID;
    out->budget = srv->budget;
    out->used = srv->used;
    out->peak = srv->peak;
    out->queued = srv->queue.size();
    out->running = running_of(srv);
    out->finished = srv->nfinished;
    out->admitted = srv->admitted;
    uint64_t total = srv->kernel_launches;
    for (const Slot& sl : srv->slots) {
        uint64_t l = 0;
        if (sl.ctx) mdg_ctx_launch_count(sl.ctx, &l);
        total += l;
    }
    std::vector<mdg_ctx*> ctxs(srv->feed_ctx, srv->feed_ctx + kSoloGens);
    ctxs.push_back(srv->alloc_ctx);
    for (mdg_ctx* c : ctxs) {
        uint64_t l = 0;
        if (c) mdg_ctx_launch_count(c, &l);
        total += l;
    }
    out->launches = total;
    out->host_admit_s = srv->admit_s;
    out->host_graph_s = srv->graph_s;
    out->host_retire_s = srv->retire_s;
    out->rechecked = srv->rechecked;
    out->host_detail_s[0] = srv->end_s;
    out->host_detail_s[1] = srv->download_s;
    out->host_detail_s[2] = srv->graph_destroy_s;
    out->host_detail_s[3] = srv->release_s;
    // the fused kernel's blocks (host-mapped flags) and the slots feeding it
    out->live_blocks = out->busy_blocks = 0;
    if (srv->q)
        for (int gen = 0; gen < kSoloGens; ++gen)
            for (int b = 0; b < srv->blocks; ++b) {
                const uint32_t f = srv->q->live[gen][b];
                out->live_blocks += f ? 1 : 0;
                out->busy_blocks += f == 2u ? 1 : 0;
            }
    out->block_slots = out->alloc_slots = 0;
    for (const Slot& sl : srv->slots) {
        out->block_slots += (sl.req && sl.state == BLOCK) ? 1 : 0;
        out->alloc_slots += (sl.req && sl.state == ALLOC) ? 1 : 0;
    }
    out->kernel_launches = srv->kernel_launches;
    return MDG_OK;
}

int mdg_server_clock(mdg_server* srv, double* t) {
    if (!srv || !t) return MDG_ERR_INVALID;
    *t = srv->now();
    return MDG_OK;
}

}  // extern "C"
