/*
 * mdref — CPU oracle for the MDcraft per-step MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of MDcraft's
 * linked-cell Verlet list, LJsCut / EAM potentials (Single and Multi solvers,
 * Periodic ghost boundary) and velocity-Verlet stepper. It is used by the
 * tests as the parity checker and by bench.py as the timed CPU baseline
 * ("port"). The product (libmdg, mdcraft_gb300) never links or calls it.
 *
 * Parity is pinned against the golden values of the reference's own C++ tests
 * (test/cxx/solver/test_argon_ball_md.cxx, test_aluminum_bulk_eam.cxx,
 * test_ljs_cut.cxx, test/cxx/neibs/test_verlet_list.cxx, test_grid.cxx,
 * test/cxx/domain/test_domain.cxx) in tests/test_oracle_golden.py.
 *
 * All arithmetic is FP64 with the reference's operation order; build with
 * -ffp-contract=off so that no FMA contraction changes rounding.
 */
#ifndef MDREF_H
#define MDREF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (same values as include/mdg.h). */
#define MDREF_OK 0
#define MDREF_ERR_INVALID (-1)
#define MDREF_ERR_NOMEM (-2)
#define MDREF_ERR_RANGE (-4)

/* mdcraft::data::Atom, 208 bytes (mdcraft/data/atom.h:21-40). V is stored
 * column-major like Eigen::Matrix<double,3,3>. */
typedef struct md_atom {
    double r[3];
    double v[3];
    double f[3];
    double V[9];
    double m, rcut, rns, Ep, Em, nc;
    uint16_t bc, kind;
    uint32_t uid;
    uint16_t tag;
    uint16_t _pad[3];
} md_atom;

/* mdcraft::lattice::Domain (mdcraft/lattice/domain.h:77-189). */
typedef struct md_domain {
    double bmin[3], bmax[3], size[3];
    int periodic[3];
    int dim;
} md_domain;

void md_domain_init(md_domain* d, double xmin, double xmax, double ymin,
                    double ymax, double zmin, double zmax);
void md_domain_fit_in_period(const md_domain* d, double v[3]);
void md_domain_shortest(const md_domain* d, double v[3]);
double md_domain_nearest_distance(const md_domain* d, const double v[3],
                                  int axis);
int md_domain_belong(const md_domain* d, const double v[3]);

/* mdcraft::neibs::Grid (mdcraft/neibs/grid.h:55-185). */
typedef struct md_grid {
    int domain_num_cells[3];
    double cell_sizes[3];
    int grid_offset[3];
    int num_cells[3];
    double min_coords[3], max_coords[3];
} md_grid;

void md_grid_build(md_grid* g, const md_domain* d, const md_atom* atoms,
                   size_t n);
void md_grid_local_index3D(const md_grid* g, const md_domain* d,
                           const double v[3], int out[3]);
int md_grid_cell_index(const md_grid* g, const int ijk[3]);
int md_grid_cells_number(const md_grid* g);
double md_grid_cell_size(const md_grid* g);
/* Writes up to 27 cell ids (padded with -1) and is_edge[3]; returns count. */
int md_grid_adjacent_cells(const md_grid* g, const md_domain* d,
                           const double r[3], int cells[27], int is_edge[3]);

/* mdcraft::neibs::VerletList (mdcraft/neibs/verlet-list.h:134-470). */
typedef struct md_nlist md_nlist;

md_nlist* md_nlist_create(size_t n, int half, int nthreads, int* status);
void md_nlist_destroy(md_nlist* nl);
/* VerletList::update(kbuf): mutates atoms' r (fit_in_period) and, for
 * kbuf > 0, rns. Returns MDREF_ERR_RANGE (and clamps) when an atom falls
 * outside the local grid, where the reference has undefined behaviour. */
int md_nlist_update(md_nlist* nl, const md_domain* d, md_atom* atoms,
                    size_t n, double kbuf);
int md_nlist_decide(const md_nlist* nl, const md_domain* d,
                    const md_atom* atoms, size_t n);
size_t md_nlist_count(const md_nlist* nl, size_t i);
const uint64_t* md_nlist_list(const md_nlist* nl, size_t i);
size_t md_nlist_total(const md_nlist* nl);
/* CSR export: offsets[n+1], idx[total] (list order as built). */
void md_nlist_export(const md_nlist* nl, uint64_t* offsets, uint64_t* idx);
/* VerletList::list_for(x): neighbours of a query point. Returns count. */
size_t md_nlist_list_for(const md_nlist* nl, const md_domain* d,
                         const md_atom* atoms, const double x[3],
                         uint64_t* out, size_t cap);
void md_nlist_grid(const md_nlist* nl, md_grid* out);
/* VerletList::sort(atoms): wraps atoms in place; sorted[] lists them by
 * owning cell (x fastest), ascending index inside a cell. */
int md_sort_atoms(const md_domain* d, md_atom* atoms, size_t n, md_atom* sorted);

/* Potentials (mdcraft/solver/potential). MD_POT_PAIR is LJsCut and
 * MD_POT_TAB the tabulated Pair; both are potential::type::pair in the
 * reference (one force stage, no density). */
#define MD_POT_PAIR 1
#define MD_POT_EAM 2
#define MD_POT_TAB 3
#define MD_POT_LJS 4

typedef struct md_pot md_pot;

md_pot* md_pot_ljcut_create(double a, double s, double rcut);
md_pot* md_pot_eam_create(double rcut, const double* Femb, const double* Rho,
                          const double* Vpar, int Nr1, double dr, int Nrh1,
                          double drh);
/* Pair(Rcutoff, Vpar, Nr1, dr) (mdcraft/solver/potential/pair.cxx:15-33):
 * Vpar = r*phi(r) on a uniform grid of step dr. */
md_pot* md_pot_pair_create(double rcut, const double* Vpar, int Nr1,
                           double dr);
/* LJs(aVr, rVr, Rcutoff) (mdcraft/solver/potential/LJs.cxx:7-29): 4 aVr
 * [(rVr/r)^12 - (rVr/r)^6] with a cubic in X = (r/rVr)^2 - 2^(1/3) that
 * takes force and energy to zero at the cutoff. */
md_pot* md_pot_ljs_create(double aVr, double rVr, double rcut);
void md_pot_destroy(md_pot* p);
double md_pot_rcut(const md_pot* p);
int md_pot_type(const md_pot* p);
/* Spline knot slopes computed by the tridiagonal sweep (EAM.cxx:603-686). */
void md_eam_init_spline(const double* y, double* z, double H1, size_t N,
                        int ib);
/* Copies the knot-slope tables (sizes Nr1, Nr1, Nrh1). */
void md_eam_slopes(const md_pot* p, double* dVpar, double* dRho,
                   double* dFemb);
/* Potential::value on squared distances (EAM, Pair, LJs; 0 for LJsCut). */
void md_pot_values(const md_pot* p, const double* r2, size_t n, double* u);
/* Embedding F and F' for one density value (EAM.cxx:562-601). */
void md_eam_embedding(const md_pot* p, double rho, double* F, double* dF);

/* Solvers: Single (mdcraft/solver/single.cxx) and Multi (multi.cxx), with the
 * Periodic boundary (boundary/periodic.cxx) or the no-op boundary. */
typedef struct md_solver md_solver;

md_solver* md_solver_single(md_pot* p, const md_domain* periodic_domain,
                            int nthreads);
md_solver* md_solver_multi(int nkinds, const md_domain* periodic_domain,
                           int nthreads);
int md_solver_add_potential(md_solver* s, int i, int j, md_pot* p);
void md_solver_destroy(md_solver* s);
int md_solver_num_stages(const md_solver* s);
void md_solver_prepare(md_solver* s, md_atom* atoms, size_t n);
void md_solver_charge(md_solver* s, md_atom* atoms, size_t n,
                      const md_nlist* nl);
void md_solver_forces(md_solver* s, md_atom* atoms, size_t n,
                      const md_nlist* nl);
void md_solver_virials(md_solver* s, md_atom* atoms, size_t n,
                       const md_nlist* nl);
/* Runs solver.stages in order (Single: [forces] or [charge, forces]). */
void md_solver_stages(md_solver* s, md_atom* atoms, size_t n,
                      const md_nlist* nl);

/* thermostat::Langevin (mdcraft/solver/thermostat/langevin.cxx:8-42) and
 * thermostat::Compound (compound.h): a list of Langevin terms applied in
 * order after each atom's own forces and before its ghost pass
 * (mdcraft/solver/pair.cxx:72-86). The reference draws from an unseeded
 * std::default_random_engine; here the normals come from Philox4x32-10
 * (Salmon et al., SC'11) keyed by `seed`, counter = {atom index, call
 * number, term index, 0}, through the Box-Muller transform, so that a run
 * is reproducible and the product can be checked draw for draw. */
typedef struct md_langevin {
    double beta, temperature, time_step;
    double heat[3], U[3];
    double xmin, xmax;
    uint64_t seed;
} md_langevin;

typedef struct md_thermo md_thermo;
md_thermo* md_thermo_create(void);
int md_thermo_add(md_thermo* t, const md_langevin* term);
void md_thermo_destroy(md_thermo* t);
/* Attaches (or with NULL detaches) the thermostat; the solver's call
 * counter restarts at `calls`. */
void md_solver_set_thermostat(md_solver* s, md_thermo* t, uint32_t calls);
uint32_t md_solver_thermo_calls(const md_solver* s);

/* Philox4x32-10 block and the three normals of one draw (exposed for the
 * known-answer test and the statistics tests). */
void md_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                      uint32_t out[4]);
void md_langevin_normals(uint64_t seed, uint32_t atom, uint32_t call,
                         uint32_t term, double z[3]);

/* stepper::Verlet::make_step (mdcraft/solver/stepper/verlet.cxx:36-85). */
void md_verlet_make_step(md_solver* s, md_atom* atoms, size_t n,
                         const md_nlist* nl, double dt);

/* Driver loop of the CPU baseline: `steps` x { make_step; if decide(): update(-1) }.
 * Returns the number of rebuilds, or a negative status. */
long md_run(md_solver* s, md_atom* atoms, size_t n, md_nlist* nl,
            const md_domain* d, double dt, long steps);

/* Totals of measure_state (test/cxx/support/md_test_utils.h:214-239):
 * out = {Ep, Em, KE, Etot, virial trace, vcom_x, vcom_y, vcom_z}. */
void md_measure_state(const md_atom* atoms, size_t n, double out[8]);

int md_hardware_threads(void);

#ifdef __cplusplus
}
#endif
#endif
