/*
 * mdg.h — C-ABI of the GB300-native MD step engine (libmdg.so).
 *
 * Drop-in boundary for MDcraft's per-step hot path on one periodic or open
 * domain: linked-cell binning + Verlet list (mdcraft/neibs), LJsCut and
 * two-pass EAM forces through the Single / Multi solvers with the Periodic
 * boundary (mdcraft/solver), and velocity-Verlet (mdcraft/solver/stepper).
 * Each entry point names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an int status: MDG_OK (0) or a negative MDG_ERR_*.
 *    mdg_last_error() returns a message for the calling thread's last error.
 *  - Units are MDcraft's: nm, ps, g/mol, kJ/mol.
 *  - Atoms cross the boundary in MDcraft's 208-byte Atom layout
 *    (mdcraft/data/atom.h:21-40) or as plain SoA double arrays, always in
 *    the caller's atom order. Internally atoms are kept cell-sorted on the
 *    device; indices returned by the API are caller indices.
 *  - Calls on one system are stream-ordered on that system's context
 *    stream; a handle may be used by one host thread at a time.
 *  - There is no CPU fallback: creating a context without a usable CUDA
 *    device fails with MDG_ERR_NODEV.
 */
#ifndef MDG_H
#define MDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDG_OK 0
#define MDG_ERR_INVALID (-1)  /* bad argument or call order */
#define MDG_ERR_NOMEM (-2)    /* device or host allocation failed */
#define MDG_ERR_OVERFLOW (-3) /* neighbour capacity exceeded (internal retry failed) */
#define MDG_ERR_RANGE (-4)    /* atom outside the grid, or table range (results flagged) */
#define MDG_ERR_TIMEOUT (-5)  /* bounded device wait expired */
#define MDG_ERR_CUDA (-6)     /* CUDA runtime error */
#define MDG_ERR_STATE (-7)    /* object not ready (e.g. forces before a list) */
#define MDG_ERR_NODEV (-8)    /* no CUDA device */
#define MDG_ERR_IO (-9)       /* potential file could not be read */

/* Arithmetic of the force stages. */
#define MDG_PREC_FP64 0  /* reference arithmetic in FP64 (parity form) */
#define MDG_PREC_MIXED 1 /* FP32 pair math, compensated FP32 sums, FP64 state */

typedef struct mdg_ctx mdg_ctx;
typedef struct mdg_system mdg_system;
typedef struct mdg_potential mdg_potential;
typedef struct mdg_thermostat mdg_thermostat;
typedef struct mdg_solver mdg_solver;

/* mdcraft::data::Atom, 208 bytes, V column-major (Eigen 3x3). */
typedef struct mdg_atom {
    double r[3];
    double v[3];
    double f[3];
    double V[9];
    double m, rcut, rns, Ep, Em, nc;
    uint16_t bc, kind;
    uint32_t uid;
    uint16_t tag;
    uint16_t _pad[3];
} mdg_atom;

/* mdcraft::lattice::Domain (mdcraft/lattice/domain.h:84-108):
 * box [bmin, bmax] and per-axis periodic flags. */
typedef struct mdg_domain {
    double bmin[3];
    double bmax[3];
    int32_t periodic[3];
} mdg_domain;

/* Totals of the reference's measure_state (test/cxx/support/md_test_utils.h:214-239). */
typedef struct mdg_state {
    double Ep, Em, KE, Etot, virial;
    double vcom[3];
} mdg_state;

const char* mdg_last_error(void);
const char* mdg_version(void);

/* ---- context ---------------------------------------------------------- */
/* One CUDA device and one stream. No reference counterpart (the reference
 * runs on host threads, mdcraft/tools/threads.h:28-221). */
int mdg_ctx_create(int device, mdg_ctx** out);
int mdg_ctx_destroy(mdg_ctx* ctx);
int mdg_ctx_synchronize(mdg_ctx* ctx);
/* The context's cudaStream_t (as void*), for callers that order their own
 * work or timing events after the engine's. */
int mdg_ctx_stream(mdg_ctx* ctx, void** stream);
/* Kernels this context has launched since creation (bench bookkeeping). */
int mdg_ctx_launch_count(mdg_ctx* ctx, uint64_t* out);
/* Per-stage device timing with CUDA events on the context stream (no
 * reference counterpart). While on, the step loop brackets each stage's
 * kernel with events; mdg_ctx_stage_time sums their elapsed times.
 * which: 0 drift, 1 density (EAM charge), 2 forces, 3 kick, 4 list rebuild. */
#define MDG_TIME_DRIFT 0
#define MDG_TIME_DENSITY 1
#define MDG_TIME_FORCES 2
#define MDG_TIME_KICK 3
#define MDG_TIME_REBUILD 4
int mdg_ctx_set_timing(mdg_ctx* ctx, int on);
int mdg_ctx_stage_time(mdg_ctx* ctx, int which, double* total_ms, uint64_t* launches);

/* ---- systems: device-resident atoms ------------------------------------ */
/* Replaces the caller-owned `Atoms` vector + `Domain` pair that every
 * reference class binds (mdcraft/data/atom.h:40, mdcraft/lattice/domain.h:84). */
int mdg_system_create(mdg_ctx* ctx, const mdg_domain* domain, size_t n,
                      mdg_system** out);
int mdg_system_destroy(mdg_system* sys);
int mdg_system_size(mdg_system* sys, size_t* n);
/* Upload/download all fields in the 208-byte Atom layout, caller order. */
int mdg_system_upload_atoms(mdg_system* sys, const mdg_atom* atoms, size_t n);
int mdg_system_download_atoms(mdg_system* sys, mdg_atom* atoms, size_t n);
/* SoA fast paths: xyz arrays are n*3 doubles, caller order. */
int mdg_system_set_positions(mdg_system* sys, const double* xyz);
int mdg_system_get_positions(mdg_system* sys, double* xyz);
int mdg_system_set_velocities(mdg_system* sys, const double* xyz);
int mdg_system_get_velocities(mdg_system* sys, double* xyz);
int mdg_system_get_forces(mdg_system* sys, double* xyz);

/* ---- Verlet list -------------------------------------------------------- */
/* VerletList::update(kbuf) (mdcraft/neibs/verlet-list.cxx:41-55): wraps
 * positions into the periodic box, rebuilds the linked-cell grid
 * (grid.cxx:43-95) and the full (half=0) or half list, snapshots positions.
 * kbuf > 0 first resets rns = kbuf * max(rcut_i + rcut_j) over the current
 * list (verlet-list.cxx:72-92). Half lists (j >= i in caller order,
 * verlet-list.cxx:345) run in the FP64 form: pair-type potentials act on
 * both atoms of a pair, EAM on its half, as the reference does; the mixed
 * form refuses them. The run loops rebuild the list of the kind last built.
 * Returns MDG_ERR_RANGE when an atom lies outside the grid (the reference
 * indexes out of bounds there); the atom is clamped into the nearest cell. */
int mdg_nlist_update(mdg_system* sys, double kbuf, int half);
/* VerletList::decide (verlet-list.cxx:110-158): *need = 1 when a rebuild is
 * due (size/uid/rcut/rns changed, or a half-skin displacement). */
int mdg_nlist_decide(mdg_system* sys, int* need);
/* Number of entries of the whole list, self entries included
 * (verlet-list.cxx:345-348 lists each atom as its own neighbour). */
int mdg_nlist_total(mdg_system* sys, size_t* total);
/* VerletList::get() as CSR in caller order: offsets[n+1], idx[total]. Each
 * atom's entries are sorted ascending (the set equals the reference's). */
int mdg_nlist_export(mdg_system* sys, uint64_t* offsets, uint64_t* idx,
                     size_t cap);
/* VerletList::sort(atoms) (verlet-list.cxx:237-249): wraps `atoms` into the
 * period in place (put_atoms_in_cells, verlet-list.cxx:176-199) and writes to
 * `sorted` (n records, not aliasing `atoms`) the same records ordered by the
 * index of their owning cell on the grid built from them (Grid::cell_index,
 * grid.cxx:134-136, x fastest), atoms of a cell in ascending input order (the
 * reference compares cells only, grid.h:31-33, so its order inside a cell is
 * unspecified). Runs on the system's device and domain; the system's atoms,
 * list and grid are not changed (the reference's sort replaces the grid that
 * later list_for calls use). MDG_ERR_RANGE: an atom lay outside the grid and
 * was sorted into the nearest cell (the reference's behaviour is undefined). */
int mdg_nlist_sort(mdg_system* sys, mdg_atom* atoms, size_t n, mdg_atom* sorted);
/* VerletList::list_for(x) (verlet-list.cxx:251-276). */
int mdg_nlist_list_for(mdg_system* sys, const double x[3], uint64_t* out,
                       size_t cap, size_t* count);
/* Grid geometry of the last rebuild (Grid members, grid.h:154-180):
 * ints = {domain_num_cells[3], grid_offset[3], num_cells[3]},
 * dbls = {cell_sizes[3]}. */
int mdg_nlist_grid(mdg_system* sys, int32_t ints[9], double dbls[3]);
/* Grid::build (grid.cxx:43-95, find_bounds grid.cxx:209-243) over the
 * system's atoms, without a list: the same geometry as mdg_nlist_grid,
 * from a bounds pass on the device (positions are wrapped into the period
 * as by a rebuild), which replaces the grid mdg_nlist_grid and
 * mdg_nlist_list_for report until the next rebuild. ints/dbls as for
 * mdg_nlist_grid; no atoms give the reference's empty grid (grid.cxx:26-34:
 * one domain cell per axis, offset 1, no local cells). */
int mdg_grid_build(mdg_system* sys, int32_t ints[9], double dbls[3]);
/* Rebuilds performed by mdg_run / mdg_nlist_update since creation. */
int mdg_nlist_rebuilds(mdg_system* sys, uint64_t* count);

/* ---- potentials ----------------------------------------------------------- */
/* LJsCut(a, s, rcut) (mdcraft/solver/potential/LJs-cut.h:15-19). */
int mdg_pot_ljcut_create(double a, double s, double rcut, mdg_potential** out);
/* EAM(rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh) (EAM.h:13-21): tables of
 * F(rho), rho(r) and r*phi(r); knot slopes are built with the reference's
 * tridiagonal sweep (EAM.cxx:603-686). */
int mdg_pot_eam_create(double rcut, const double* Femb, const double* Rho,
                       const double* Vpar, int Nr1, double dr, int Nrh1,
                       double drh, mdg_potential** out);
/* EAM(std::string filename) (EAM.cxx:55-87): single-element setfl file;
 * unlike the reference, a missing or short file fails with MDG_ERR_IO. */
int mdg_pot_eam_create_from_file(const char* path, mdg_potential** out);
/* LJs(aVr, rVr, Rcutoff) (mdcraft/solver/potential/LJs.h:14-18): Lennard-
 * Jones 4 aVr [(rVr/r)^12 - (rVr/r)^6] with a cubic in X = (r/rVr)^2 - 2^(1/3)
 * that brings force and energy to zero at the cutoff (LJs.cxx:7-29). */
int mdg_pot_ljs_create(double aVr, double rVr, double rcut, mdg_potential** out);
/* Pair(Rcutoff, Vpar, Nr1, dr) (mdcraft/solver/potential/pair.h:13-18,
 * pair.cxx:15-33): tabulated r*phi(r) with the reference's spline; pair
 * energy phi(r)/2 per side, force from d(r*phi)/dr. */
int mdg_pot_pair_create(double rcut, const double* Vpar, int Nr1, double dr,
                        mdg_potential** out);
/* Pair(std::string filename) (pair.cxx:36-56): skips 4 lines, reads
 * `Nr1 dr rcut` and Nr1 values of r*phi in eV*A; a missing or short file
 * fails with MDG_ERR_IO. */
int mdg_pot_pair_create_from_file(const char* path, mdg_potential** out);
int mdg_pot_destroy(mdg_potential* pot);
/* Base::rcut() (mdcraft/solver/potential/base.h:37). */
int mdg_pot_rcut(mdg_potential* pot, double* rcut);
/* Potential::value(r2[], U[], n) (EAM.cxx:141-174, pair.cxx:81-114,
 * LJs.cxx:61-71; the Python bindings' value(), _potential.cxx:88-201): the
 * pair energy term of each squared distance (V(r)/2r for the tabulated
 * types, 0 past the table), with no cutoff test, as the reference; LJsCut
 * keeps the base class's value (base.cxx:19) and gives 0. Host arrays of n
 * doubles; evaluated on ctx's device with the FP64 bodies of the force
 * kernels. */
int mdg_pot_values(mdg_ctx* ctx, mdg_potential* pot, const double* r2, size_t n, double* u);
/* EAM::embeddingEnergy(rho[], F[], dF[], n) (EAM.cxx:562-601): F(rho) and
 * F'(rho) (dF may be NULL). Densities outside the table take the reference's
 * extrapolation, with its output array read as zero. MDG_ERR_INVALID for a
 * potential without an embedding table (LJsCut, LJs, Pair). */
int mdg_pot_embedding(mdg_ctx* ctx, mdg_potential* pot, const double* rho, size_t n, double* F,
                      double* dF);
/* The per-atom overloads of Potential (potential/base.h:44-56):
 * force(atom, neibs, nlist) (LJs-cut.cxx:22-68, EAM.cxx:465-497),
 * virial(atom, neibs, nlist) (LJs-cut.cxx:70-131, EAM.cxx:306-354) and
 * density(atom, neibs, nlist) (EAM.cxx:541-560) of one atom over an explicit
 * list of indices into neibs[0..nneibs), in the list's order with the
 * reference's FP64 arithmetic, on ctx's device. Pairs use raw differences
 * r_j - r_i (no periodic images), as the reference's per-atom calls do.
 * `atom` may point into neibs. With half != 0, LJsCut also pushes each
 * pair's force (force) and energy and virial (virial) onto the neighbour;
 * EAM ignores it, as the reference does. The records are updated in place:
 * f (force), V, Ep and, for EAM, Em (virial), nc (density). LJs and Pair
 * are not supported here (MDG_ERR_INVALID), nor is density for LJsCut. */
#define MDG_ATOM_FORCE 0
#define MDG_ATOM_VIRIAL 1
#define MDG_ATOM_DENSITY 2
int mdg_pot_atom(mdg_ctx* ctx, mdg_potential* pot, int what, mdg_atom* atom, mdg_atom* neibs, size_t nneibs,
                 const uint64_t* list, size_t count, int half);

/* ---- solvers ------------------------------------------------------------------- */
/* Single(pot, boundary) (mdcraft/solver/single.h:37-42). periodic != 0
 * selects boundary::Periodic(domain) (boundary/periodic.h:29), else the
 * no-op boundary. */
int mdg_solver_single(mdg_potential* pot, int periodic, mdg_solver** out);
/* Multi(boundary, thermostat, nkinds) (mdcraft/solver/multi.h:42-47). */
int mdg_solver_multi(int nkinds, int periodic, mdg_solver** out);
/* Multi::add_potential(i, j, pot) (multi.cxx:28-49). */
int mdg_solver_add_potential(mdg_solver* s, int i, int j, mdg_potential* pot);
int mdg_solver_destroy(mdg_solver* s);
/* stages.size() (mdcraft/solver/isolver.h:31): 1 for pair, 2 for EAM. */
int mdg_solver_num_stages(mdg_solver* s, int* n);
int mdg_solver_set_precision(mdg_solver* s, int precision);
/* Pair::prepare / charge / forces / virials (mdcraft/solver/pair.cxx:16-114)
 * on a system whose list is built (prepare, which reads no list, also runs
 * on a system without one). */
int mdg_solver_prepare(mdg_solver* s, mdg_system* sys);
int mdg_solver_charge(mdg_solver* s, mdg_system* sys);
int mdg_solver_forces(mdg_solver* s, mdg_system* sys);
int mdg_solver_virials(mdg_solver* s, mdg_system* sys);
/* All of solver.stages in order (single.cxx:23-35). */
int mdg_solver_stages(mdg_solver* s, mdg_system* sys);

/* ---- launch shapes ------------------------------------------------------------- */
/* Launch shapes of a system's kernels, set by the project's autotuner
 * (mdcraft_gb300/tune.py: each candidate timed on the system itself, the
 * choice cached per GPU and workload); 0 restores the measured default.
 * No counterpart in the reference. Values:
 *   MDG_SHAPE_LIST_CELLS_PER_BLOCK   cells (warps) per block of the list build: 2, 4, 8
 *   MDG_SHAPE_FORCE_BLOCKS_PER_SM    register budget of the mixed force pass: 3, 4, or 8
 *                                    (eight 128-thread blocks: the step loop's EAM force
 *                                    pass; the other force passes take 4 then)
 *   MDG_SHAPE_DENSITY_BLOCKS_PER_SM  register budget of the mixed density pass: 3, 4, 5 */
#define MDG_SHAPE_LIST_CELLS_PER_BLOCK 0
#define MDG_SHAPE_FORCE_BLOCKS_PER_SM 1
#define MDG_SHAPE_DENSITY_BLOCKS_PER_SM 2
int mdg_system_set_shape(mdg_system* sys, int what, int value);
int mdg_system_get_shape(mdg_system* sys, int what, int* value);

/* ---- thermostats ------------------------------------------------------------ */
/* thermostat::Langevin(beta, temperature, time_step, heat_x, heat_y, heat_z,
 * Ux, Uy, Uz, xmin, xmax) (mdcraft/solver/thermostat/langevin.h:17-29):
 * during the force stage each atom with xmin <= x <= xmax gets
 * f += heat * (sqrt(m) * N(0, sigma) - (v - U) * beta * m),
 * sigma = sqrt(2 beta Kb T / time_step) (langevin.cxx:21-42). The normals
 * come from Philox4x32-10 keyed by `seed` with the counter {caller index of
 * the atom, call number of the system, term index, 0} (the reference seeds
 * std::default_random_engine from std::random_device, so its runs do not
 * repeat; these do). */
typedef struct mdg_langevin {
    double beta, temperature, time_step;
    int32_t heat[3];
    int32_t _pad;
    double U[3];
    double xmin, xmax;
    uint64_t seed;
} mdg_langevin;
int mdg_thermo_langevin_create(const mdg_langevin* params, mdg_thermostat** out);
/* Langevin::set_friction / set_temperature / set_average_velocity /
 * set_heating_axes / set_dimensions (langevin.cxx:44-76) in one call, and
 * the getters friction() ... xmax() (langevin.cxx:78-82). */
int mdg_thermo_langevin_set(mdg_thermostat* t, const mdg_langevin* params);
int mdg_thermo_langevin_get(mdg_thermostat* t, mdg_langevin* params);
/* thermostat::Compound (mdcraft/solver/thermostat/compound.h:12-24): its
 * parts apply in the order they were added. */
int mdg_thermo_compound_create(mdg_thermostat** out);
int mdg_thermo_compound_add(mdg_thermostat* compound, mdg_thermostat* part);
int mdg_thermo_destroy(mdg_thermostat* t);
/* The thermostat argument of Single / Multi (single.h:37-42, multi.h:42-47);
 * NULL restores the no-op thermostat. The solver keeps the pointer. */
int mdg_solver_set_thermostat(mdg_solver* s, mdg_thermostat* t);
/* Thermostat applications on this system so far (the Philox call number
 * of the next one), and a way to set it (to resume a run). */
int mdg_system_thermo_calls(mdg_system* sys, uint32_t* calls);
int mdg_system_set_thermo_calls(mdg_system* sys, uint32_t calls);

/* ---- stepper ----------------------------------------------------------------------- */
/* stepper::Verlet::make_step(atoms, nlist, dt) (verlet.cxx:36-48). */
int mdg_verlet_make_step(mdg_solver* s, mdg_system* sys, double dt);
/* Driver loop, fused on the device: `steps` x { make_step(dt); if decide():
 * update(-1) }, the loop of the reference's drivers
 * (test/python/solver/test-EAM.py:158-200). The rebuild test is read back
 * while the force kernels of the same step run. */
int mdg_run(mdg_solver* s, mdg_system* sys, double dt, long steps);
/* Same loop, end to end from host buffers: uploads positions and velocities
 * (n*3 doubles each, caller order), runs `steps`, and downloads positions,
 * velocities and forces. */
int mdg_run_host(mdg_solver* s, mdg_system* sys, double dt, long steps,
                 double* pos, double* vel, double* force);

/* ---- measurement ---------------------------------------------------------------- */
/* FP64 device reduction of measure_state (md_test_utils.h:214-239). Uses
 * the per-atom Ep, Em, V of the last mdg_solver_virials call. */
int mdg_system_measure(mdg_system* sys, mdg_state* out);
/* The reduction of mdg_system_measure on device arrays the caller owns,
 * allocating nothing: for callers that cannot call cudaMalloc (code running
 * under another component's device-memory pool, latency-critical loops that
 * cannot afford an allocation's synchronisation, plug-in hosts that only
 * hand out pre-registered buffers). No counterpart in the reference.
 * Inputs (device, FP64, n atoms): d_m[n]; d_v[3n] = vx|vy|vz; d_Ep[n];
 * d_Em[n]; d_V[9n] = the nine virial components, component-major. Output:
 * d_out[8] (device) = {Ep, Em, KE, Etot, virial trace, vcom x, y, z}.
 * Launches on `stream` (a cudaStream_t; NULL = default stream) and does not
 * synchronise. Scratch is a static device array of 256 KB held by every GPU
 * that loads the library: at most 8,388,608 atoms per call (larger n fails
 * with MDG_ERR_INVALID); calls whose kernels overlap on the GPU race on it.
 * The first call on a device looks the array up (cudaGetSymbolAddress),
 * which with lazy module loading (the CUDA default) also loads the module
 * and can synchronise: make that first call at set-up, as a warm-up, before
 * any stream capture. An error already pending from an earlier CUDA call is
 * returned without launching anything. */
int mdg_measure_static(const double* d_m, const double* d_v, const double* d_Ep, const double* d_Em,
                       const double* d_V, size_t n, double* d_out, void* stream);
/* Error/diagnostic flags accumulated on the device since the last call
 * (bit 0 atom out of grid, bit 1 neighbour overflow, bit 2 EAM table range,
 * bit 3 non-finite force, bit 4 a listed pair whose image lies more than one
 * cell from the atom's cell: the mixed form's pair vector cannot express it.
 * Bit 4 is a guard: a listed pair is within rns, which is at most one cell
 * edge, so it is not raised by any input); clears them. */
int mdg_system_flags(mdg_system* sys, uint32_t* flags);

/* ---- serving: continuous batching of independent systems ------------------------
 * No counterpart in the reference, whose drivers run one system per process
 * (test/python/solver/test-EAM.py:101-200). A server keeps up to `slots`
 * systems resident on one GPU, each on its own stream running its whole
 * driver loop (mdg_run) as one graph launch, so the work of different
 * requests overlaps on the device. A request (atoms, domain, solver, dt,
 * steps) waits in a FIFO until a slot is free and its device footprint fits
 * in the budget left by the running ones; when it finishes its slot and
 * memory go to the next. System memory comes stream-ordered from a pool
 * owned by the server, so admitting and retiring a request never waits for
 * the whole device. Results do not depend on what else runs: every kernel
 * reads only its own system, in a fixed order. A server is used by one host
 * thread at a time; the solvers it is given must outlive their requests. */
typedef struct mdg_server mdg_server;

typedef struct mdg_server_config {
    int slots;          /* systems on the GPU at once (>= 1) */
    size_t hbm_budget;  /* device bytes the live systems may hold; 0 = half the free memory */
    size_t max_atoms;   /* largest request accepted (sizes the pinned staging) */
    int block_threads;  /* fused one-block loop per system (mixed precision, one kind,
                           <= 65536 atoms): its threads (256, 512, 640, 768, 896, 1024), 0 = the default
                           (768), -1 = off (a graph loop per request instead) */
    int order;          /* admission order of waiting requests: MDG_ORDER_FIFO (0, the
                           default), MDG_ORDER_LARGEST (most atom-steps first, which
                           shortens the tail of a backlog at the cost of small requests'
                           latency) or MDG_ORDER_BALANCED (arrival order, except that the
                           largest waiting request goes first once its atom-steps reach
                           the waiting atom-steps per worker, a block of the fused loop or
                           else a slot: largest-first for the end of a backlog only) */
} mdg_server_config;
#define MDG_ORDER_FIFO 0
#define MDG_ORDER_LARGEST 1
#define MDG_ORDER_BALANCED 2

typedef struct mdg_request_info {
    int status;         /* MDG_OK or the error that ended the request */
    int done;           /* 1 once the result is available */
    double t_submit;    /* server clock (s): submitted, admitted to a slot, finished */
    double t_admit;
    double t_done;
    uint64_t rebuilds;  /* list rebuilds during the run */
    size_t footprint;   /* device bytes the request held */
    double service_s;   /* time the request ran, without its queueing: for a fused
                           one-block run, from the block's start on it to its
                           completion record (GPU clock); for a graph loop, from
                           its admission to completion (server clock) */
} mdg_request_info;

typedef struct mdg_server_stats {
    size_t budget, used, peak; /* device bytes: budget, held now, most held at once */
    size_t queued, running, finished;
    uint64_t admitted;
    uint64_t launches;  /* kernels launched for all requests so far */
    double host_admit_s;  /* host seconds spent admitting (set-up, first list, graph) */
    double host_graph_s;  /* of which capturing and instantiating step-loop graphs */
    double host_retire_s; /* host seconds spent retiring (result copy, release) */
    uint64_t rechecked;   /* requests repeated on the checked path (first list outgrew its sizing) */
    double host_detail_s[4]; /* of retiring: run bookkeeping, result gather, graph release, memory release */
    size_t live_blocks;   /* blocks of the fused loop's kernel alive now, over all its launches in
                             flight (running, waiting for a request, or launched and not yet resident) */
    size_t busy_blocks;   /* of which running a request */
    size_t block_slots;   /* requests published to the fused loop and not yet finished */
    size_t alloc_slots;   /* requests admitted whose buffers are still being allocated */
    uint64_t kernel_launches; /* launches of the fused loop's kernel so far */
} mdg_server_stats;

int mdg_server_create(int device, const mdg_server_config* cfg, mdg_server** out);
/* Waits for running requests, then frees everything. */
int mdg_server_destroy(mdg_server* srv);
/* Queues a request; copies the atoms (caller order, 208 B records). The
 * solver's precision at submission is used. Fails with MDG_ERR_NOMEM when
 * the request alone would exceed the budget and MDG_ERR_INVALID when n >
 * max_atoms. Does not wait for the device. */
int mdg_server_submit(mdg_server* srv, mdg_solver* solver, const mdg_domain* domain, const mdg_atom* atoms,
                      size_t n, double dt, long steps, uint64_t* id);
/* Retires finished requests and admits queued ones; does not block on
 * running work. `running` (optional) gets the number of busy slots. */
int mdg_server_progress(mdg_server* srv, size_t* running);
/* progress(), then hands out up to `cap` ids of requests finished since the
 * last poll. */
int mdg_server_poll(mdg_server* srv, uint64_t* ids, size_t cap, size_t* count);
/* Drives progress until request `id` is finished or `timeout_s` passes
 * (MDG_ERR_TIMEOUT). */
int mdg_server_wait(mdg_server* srv, uint64_t id, double timeout_s);
/* Copies a finished request's atoms (positions, velocities, forces after
 * the last step; caller order) and its record, then forgets the request.
 * `atoms` may be NULL to read only the record. MDG_ERR_STATE if it is not
 * finished. */
int mdg_server_result(mdg_server* srv, uint64_t id, mdg_atom* atoms, size_t n, mdg_request_info* info);
int mdg_server_stats_get(mdg_server* srv, mdg_server_stats* out);
/* Seconds since the server was created (the clock of mdg_request_info). */
int mdg_server_clock(mdg_server* srv, double* t);
/* Device bytes a request of n atoms with `neighbours` list entries per atom
 * is charged at admission. */
size_t mdg_server_footprint(size_t n, int neighbours);

#ifdef __cplusplus
}
#endif
#endif
