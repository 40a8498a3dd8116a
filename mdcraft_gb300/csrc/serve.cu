// serve.cu — continuous batching of independent MD systems on one GPU.
//
// The reference runs one system per process, its driver loop on the host
// (test/python/solver/test-EAM.py:101-200); there is no serving layer to
// mirror. Here a request is a whole driver loop (mdg_run: `steps` x
// make_step + decide/update) over its own system. The server owns `slots`
// streams. A slot takes the head of the FIFO when it is free and the
// request's device footprint fits in the budget left by the running ones;
// the request's system is created from the server's stream-ordered memory
// pool, its atoms uploaded, its first list built, and its loop launched as
// one graph (WHILE over steps, IF over rebuilds). Slots run concurrently,
// so small systems that fill a few SMs each share the GPU. Completion is
// found by polling one event per slot; the result is copied out and the
// system's buffers go back to the pool behind the slot's last work, with no
// device-wide synchronisation anywhere on the admit/retire path.
//
// Results are independent of the mix: every kernel reads and writes only its
// own system's buffers, sums in a fixed order and uses no atomics across
// systems, so a request gives the same bits alone or among others.
#include <algorithm>
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
};

// A slot's request goes RUN (set-up + graph loop enqueued) -> COPY (result
// gather + device-to-host copy enqueued) -> finished; each transition is
// taken when the slot's event has passed, so the host never waits.
enum SlotState { IDLE = 0, RUN = 1, COPY = 2 };

struct Slot {
    mdg_ctx* ctx = nullptr;
    cudaEvent_t ev = nullptr;
    Request* req = nullptr;
    mdg_system* sys = nullptr;
    SystemMemory mem;
    int state = IDLE;
    int checked = 0;                  // request set up on the synchronous, checked path
    DevStatus* first_status = nullptr;  // device status after the first list build (pinned)
    void* hblock = nullptr;  // pinned status words of the slot's systems
    void* pin = nullptr;     // pinned transfer staging of the slot (max_atoms records)
};

// Neighbour entries per atom the admission estimate assumes when the atoms
// give no better figure: a dense liquid or solid at rns = rc + skin.
constexpr int kDefaultNeighbours = 96;

}  // namespace

struct mdg_server {
    int device = 0;
    cudaMemPool_t pool = nullptr;
    size_t budget = 0, used = 0, peak = 0;
    size_t max_atoms = 0;
    std::vector<Slot> slots;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> reqs;
    std::deque<uint64_t> finished;
    uint64_t next_id = 1;
    uint64_t admitted = 0;
    size_t nfinished = 0;
    double admit_s = 0.0, graph_s = 0.0, retire_s = 0.0;
    uint64_t rechecked = 0;
    double graph_destroy_s = 0.0, release_s = 0.0, end_s = 0.0, download_s = 0.0;
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

void finish(mdg_server* sv, Request* r, int status) {
    r->info.status = status;
    r->info.done = 1;
    r->info.t_done = sv->now();
    sv->finished.push_back(r->id);
    sv->nfinished++;
}

void retire(mdg_server* sv, Slot& sl) {
    if (sl.sys) {
        sv->graph_s += sl.sys->graph_build_s;
        double t = sv->now();
        if (sl.sys->run_exec) cudaGraphExecDestroy(sl.sys->run_exec);
        if (sl.sys->run_graph) cudaGraphDestroy(sl.sys->run_graph);
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
}

// Sets up the request on the slot and enqueues its whole run; on failure
// the request is finished with the error and the slot freed.
void admit_impl(mdg_server* sv, Slot& sl, Request* r, int checked);

void admit(mdg_server* sv, Slot& sl, Request* r, int checked = 0) {
    double t = sv->now();
    admit_impl(sv, sl, r, checked);
    sv->admit_s += sv->now() - t;
}

void fail(mdg_server* sv, Slot& sl, int rc) {
    Request* r = sl.req;
    r->info.footprint = r->footprint;
    retire(sv, sl);
    sl.state = IDLE;
    finish(sv, r, rc);
}

void admit_impl(mdg_server* sv, Slot& sl, Request* r, int checked) {
    if (!sl.req) {
        sl.req = r;
        r->info.t_admit = sv->now();
        sv->admitted++;
        sv->used += r->footprint;
        sv->peak = std::max(sv->peak, sv->used);
    }
    sl.checked = checked;
    size_t n = r->atoms.size();
    int rc = system_create(sl.ctx, &r->dom, n, &sl.mem, &sl.sys);
    int prec_saved = r->solver->precision;
    r->solver->precision = r->precision;
    if (rc == MDG_OK && !checked) {
        // everything enqueued, nothing waited for
        rc = request_begin(r->solver, sl.sys, r->atoms.data(), r->dt, r->steps, sl.first_status);
    } else if (rc == MDG_OK) {
        // the checked path: the driver's calls one by one, each list build
        // verified (and grown) before the run goes on
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
        // charge what the system holds once its capacities are sized
        if (sl.sys->dev_bytes > r->footprint) {
            sv->used += sl.sys->dev_bytes - r->footprint;
            r->footprint = sl.sys->dev_bytes;
            sv->peak = std::max(sv->peak, sv->used);
        }
        cudaError_t e = cudaEventRecord(sl.ev, sl.ctx->stream);
        if (e != cudaSuccess) rc = cuda_status(e, "slot event");
    }
    if (rc != MDG_OK) {
        fail(sv, sl, rc);
        return;
    }
    sl.state = RUN;
}

// The slot's event has passed: advance its request one state.
void advance_impl(mdg_server* sv, Slot& sl);

void advance(mdg_server* sv, Slot& sl) {
    double t = sv->now();
    advance_impl(sv, sl);
    sv->retire_s += sv->now() - t;
}

void advance_impl(mdg_server* sv, Slot& sl) {
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
            admit_impl(sv, sl, r, 1);
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
            return;
        }
        if (!relaunched) sl.state = COPY;
        return;
    }
    // COPY: the result is in the slot's pinned staging
    memcpy(r->atoms.data(), sl.pin, r->atoms.size() * sizeof(mdg_atom));
    r->info.rebuilds = sl.sys->rebuilds;
    r->info.footprint = r->footprint;
    retire(sv, sl);
    sl.state = IDLE;
    finish(sv, r, MDG_OK);
}

int progress(mdg_server* sv) {
    MDG_CUDA(cudaSetDevice(sv->device));
    for (Slot& sl : sv->slots) {
        if (!sl.req) continue;
        cudaError_t e = cudaEventQuery(sl.ev);
        if (e == cudaErrorNotReady) continue;
        if (e != cudaSuccess) {
            fail(sv, sl, cuda_status(e, "request"));
            continue;
        }
        advance(sv, sl);
    }
    // FIFO admission: the head waits for memory rather than being overtaken
    for (Slot& sl : sv->slots) {
        if (sv->queue.empty()) break;
        if (sl.req) continue;
        Request* r = sv->queue.front();
        if (sv->used + r->footprint > sv->budget && sv->used > 0) break;
        sv->queue.pop_front();
        admit(sv, sl, r);
    }
    return MDG_OK;
}

size_t running_of(const mdg_server* sv) {
    size_t k = 0;
    for (const Slot& sl : sv->slots) k += sl.req ? 1 : 0;
    return k;
}

void server_free(mdg_server* sv) {
    cudaSetDevice(sv->device);
    for (Slot& sl : sv->slots) {
        if (sl.ctx) cudaStreamSynchronize(sl.ctx->stream);
        if (sl.sys) retire(sv, sl);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.hblock) cudaFreeHost(sl.hblock);
        if (sl.pin) cudaFreeHost(sl.pin);
        if (sl.ctx) mdg_ctx_destroy(sl.ctx);
    }
    for (auto& kv : sv->reqs) delete kv.second;
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    delete sv;
}

}  // namespace

extern "C" {

size_t mdg_server_footprint(size_t n, int neighbours) { return footprint_of(n, neighbours); }

int mdg_server_create(int device, const mdg_server_config* cfg, mdg_server** out) {
    if (!cfg || !out || cfg->slots < 1 || cfg->slots > 1024 || cfg->max_atoms == 0 || cfg->max_atoms >= kMaxAtoms)
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
    if (e != cudaSuccess) {
        int rc = cuda_status(e, "server memory");
        server_free(sv);
        return rc;
    }
    sv->slots.resize(cfg->slots);
    for (Slot& sl : sv->slots) {
        int rc = mdg_ctx_create(device, &sl.ctx);
        if (rc == MDG_OK) {
            e = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaMallocHost(&sl.hblock, 1024);
            if (e == cudaSuccess) e = cudaMallocHost(&sl.pin, cfg->max_atoms * sizeof(mdg_atom));
            if (e != cudaSuccess) rc = cuda_status(e, "slot");
        }
        if (rc != MDG_OK) {
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
    uint64_t total = 0;
    for (const Slot& sl : srv->slots) {
        uint64_t l = 0;
        if (sl.ctx) mdg_ctx_launch_count(sl.ctx, &l);
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
    return MDG_OK;
}

int mdg_server_clock(mdg_server* srv, double* t) {
    if (!srv || !t) return MDG_ERR_INVALID;
    *t = srv->now();
    return MDG_OK;
}

}  // extern "C"
