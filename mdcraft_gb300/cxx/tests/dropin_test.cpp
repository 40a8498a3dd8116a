// C++ drop-in test: MDcraft-style host code (VerletList / Single / Multi /
// EAM / LJsCut / LJs / Pair / Periodic / Langevin / stepper::Verlet, as
// test/cxx/solver/*.cxx, test/cxx/neibs/test_verlet_list.cxx and
// problems/NiAl/test-NiAl.py use them) compiled against the drop-in headers
// and linked with libmdg. Asserts the reference tests' golden values, and
// for the potentials those tests do not cover, energy conservation and the
// Langevin thermostat's temperature.
//
// usage: dropin_test <LAMMPS Ar ball file> <Al setfl EAM file> [NiAl pair file]
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>

#include <mdcraft/data/atom.h>
#include <mdcraft/lattice/domain.h>
#include <mdcraft/neibs/verlet-list.h>
#include <mdcraft/solver/boundary/periodic.h>
#include <mdcraft/solver/potential/EAM.h>
#include <mdcraft/solver/multi.h>
#include <mdcraft/solver/potential/LJs-cut.h>
#include <mdcraft/solver/potential/LJs.h>
#include <mdcraft/solver/potential/pair.h>
#include <mdcraft/solver/single.h>
#include <mdcraft/solver/thermostat/compound.h>
#include <mdcraft/solver/thermostat/langevin.h>
#include <mdcraft/solver/stepper/verlet.h>
#include <mdcraft/tools/threads.h>

using namespace mdcraft;
using data::Atom;
using data::Atoms;
using data::vector;

static int g_fail = 0, g_checks = 0;

#define CHECK_NEAR(a, b, tol)                                                                      \
    do {                                                                                           \
        ++g_checks;                                                                                \
        double a_ = (a), b_ = (b);                                                                 \
        if (!(std::fabs(a_ - b_) <= (tol))) {                                                      \
            ++g_fail;                                                                              \
            std::printf("FAIL %s:%d  %s = %.17g, expected %.17g (tol %g)\n", __FILE__, __LINE__, #a, \
                        a_, b_, (double)(tol));                                                    \
        }                                                                                          \
    } while (0)
#define CHECK(c)                                                           \
    do {                                                                   \
        ++g_checks;                                                        \
        if (!(c)) {                                                        \
            ++g_fail;                                                      \
            std::printf("FAIL %s:%d  %s\n", __FILE__, __LINE__, #c);       \
        }                                                                  \
    } while (0)

struct State {
    double Ep = 0, Em = 0, KE = 0, Etot = 0, virial = 0;
    vector vcom;
};

// measure_state (test/cxx/support/md_test_utils.h:214-239)
static State measure(const Atoms& atoms) {
    State s;
    double tm = 0.0;
    vector com = vector::Zero();
    for (const auto& a : atoms) {
        s.Ep += a.Ep;
        s.Em += a.Em;
        s.virial += a.V.trace();
        com += a.m * a.v;
        tm += a.m;
    }
    if (tm > 0) com /= tm;
    for (const auto& a : atoms) s.KE += 0.5 * a.m * (a.v - com).squaredNorm();
    s.Etot = s.Ep + s.Em + s.KE;
    s.vcom = com;
    return s;
}

// run_md_steps (md_test_utils.h:255-279)
static std::vector<State> run_md_steps(solver::Single& solver, solver::stepper::Verlet& stepper, Atoms& atoms,
                                       neibs::VerletList& nlist, double dt, int steps, int interval) {
    std::vector<State> h;
    auto recompute = [&]() {
        auto& raw = nlist.get();
        solver.prepare(atoms, atoms, raw);
        for (auto& st : solver.stages) st(atoms, atoms, raw);
        solver.virials(atoms, atoms, raw);
        return measure(atoms);
    };
    nlist.update(-1.0);
    h.push_back(recompute());
    for (int s = 1; s <= steps; ++s) {
        stepper.make_step(atoms, nlist.get(), dt);
        if (interval > 0 && s % interval == 0) nlist.update(-1.0);
        h.push_back(recompute());
    }
    return h;
}

static void set_common(Atoms& atoms, double mass, double rcut, double skin) {
    for (size_t i = 0; i < atoms.size(); ++i) {
        atoms[i].uid = atoms[i].uid == 0 ? (unsigned)(i + 1) : atoms[i].uid;
        atoms[i].kind = atoms[i].kind == 0 ? 1 : atoms[i].kind;
        atoms[i].m = mass;
        atoms[i].rcut = rcut;
        atoms[i].rns = skin * rcut;
    }
}

static void test_verlet_lists() {
    tools::Threads threads(1);
    {
        Atoms atoms(3);
        atoms[0].r << 0.20, 0.0, 0.0;
        atoms[1].r << 0.85, 0.0, 0.0;
        atoms[2].r << 2.50, 0.0, 0.0;
        for (auto& a : atoms) {
            a.rns = 0.80;
            a.rcut = 0.80;
            a.m = 1.0;
        }
        lattice::Domain domain(0.0, 3.0, -1.0, 1.0, -1.0, 1.0);
        neibs::VerletList nlist(atoms, atoms, domain, threads);
        nlist.update(-1.0);
        CHECK(nlist[0].size() == 2 && nlist[1].size() == 2 && nlist[2].size() == 1);
        CHECK(nlist[0][0] == 0 && nlist[0][1] == 1 && nlist[2][0] == 2);
    }
    {
        Atoms atoms(2);
        atoms[0].r << -0.48, 0.0, 0.0;
        atoms[1].r << 0.48, 0.0, 0.0;
        for (auto& a : atoms) {
            a.rns = 0.10;
            a.rcut = 0.10;
            a.m = 1.0;
        }
        lattice::Domain domain(-0.5, 0.5, -0.5, 0.5, -0.5, 0.5);
        domain.set_periodic(0, true);
        neibs::VerletList nlist(atoms, atoms, domain, threads);
        nlist.update(-1.0);
        CHECK(nlist[0].size() == 2 && nlist[1].size() == 2);
    }
    {
        Atoms atoms(2);
        atoms[0].r << 0.10, 0.10, 0.10;
        atoms[1].r << 0.50, 0.10, 0.10;
        for (int i = 0; i < 2; ++i) {
            atoms[i].rcut = 0.60;
            atoms[i].rns = 0.80;
            atoms[i].m = 1.0;
            atoms[i].uid = i + 1;
        }
        lattice::Domain domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0);
        neibs::VerletList nlist(atoms, atoms, domain, threads, true);
        nlist.update(-1.0);
        atoms[0].r.x() += 0.09;
        CHECK(!nlist.decide());
        atoms[0].r.x() += 0.02;
        CHECK(nlist.decide());
    }
    {
        // test/cxx/neibs/test_verlet_list.cxx:107-122 (SortOrdersAtomsByOwningCell)
        Atoms atoms(3);
        atoms[0].r << 1.60, 0.10, 0.10;
        atoms[1].r << 0.15, 0.10, 0.10;
        atoms[2].r << 0.95, 0.10, 0.10;
        for (auto& a : atoms) {
            a.rcut = 0.40;
            a.rns = 0.40;
            a.m = 1.0;
        }
        lattice::Domain domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0);
        neibs::VerletList nlist(atoms, atoms, domain, threads);
        auto sorted = nlist.sort(atoms);
        CHECK(sorted.size() == 3U);
        CHECK(sorted[0].r.x() < sorted[1].r.x() && sorted[1].r.x() < sorted[2].r.x());
    }
    {
        tools::Threads two(2);
        Atoms atoms(1);
        lattice::Domain domain(0.0, 1.0, 0.0, 1.0, 0.0, 1.0);
        bool thrown = false;
        try {
            neibs::VerletList nl(atoms, atoms, domain, two, true);
        } catch (const std::runtime_error&) {
            thrown = true;
        }
        CHECK(thrown);
    }
}

// test/cxx/solver/test_argon_ball_md.cxx
static void test_argon_ball(const std::string& path) {
    std::ifstream file(path);
    CHECK(file.is_open());
    if (!file.is_open()) return;
    std::string line;
    size_t total = 0;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    std::unordered_map<int, double> mass;
    Atoms atoms;
    bool in_atoms = false;
    while (std::getline(file, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream iss(line);
        if (!in_atoms) {
            if (line.find("atoms") != std::string::npos) iss >> total;
            for (int a = 0; a < 3; ++a) {
                const char* key[3] = {"xlo xhi", "ylo yhi", "zlo zhi"};
                if (line.find(key[a]) != std::string::npos) {
                    std::istringstream s2(line);
                    s2 >> lo[a] >> hi[a];
                }
            }
            if (line.find("Atoms") != std::string::npos) in_atoms = true;
            continue;
        }
        Atom a{};
        double x, y, z;
        if (!(iss >> a.uid >> a.kind >> x >> y >> z)) continue;
        a.r << x * 0.1, y * 0.1, z * 0.1;
        atoms.push_back(a);
        if (atoms.size() == total) break;
    }
    CHECK(atoms.size() == 130124);
    lattice::Domain domain(lo[0] * 0.1, hi[0] * 0.1, lo[1] * 0.1, hi[1] * 0.1, lo[2] * 0.1, hi[2] * 0.1);
    tools::Threads threads(1);
    solver::potential::LJsCut potential{1.03120074782442750, 0.33841043857528683, 0.8125};
    solver::Single solver{potential, solver::boundary::dummy_boundary, solver::thermostat::dummy_thermostat,
                          threads};
    solver::stepper::Verlet stepper{solver, threads};
    set_common(atoms, 40.0, potential.rcut(), 10.125 / 8.125);
    for (auto& a : atoms) a.v = vector::Zero();
    neibs::VerletList nlist(atoms, atoms, domain, threads);
    auto h = run_md_steps(solver, stepper, atoms, nlist, 4e-3, 2, 1);
    CHECK_NEAR(h[2].Ep, -1.0244383150033894e+06, 1.0e-3);
    CHECK_NEAR(h[2].virial, -1.1164231473675424e+05, 1.0e-3);
    CHECK_NEAR(h[2].Etot, h[0].Etot, 2.0);
    size_t a1 = 0, a2 = 0;
    for (size_t i = 0; i < atoms.size(); ++i) {
        if (atoms[i].uid == 1) a1 = i;
        if (atoms[i].uid == 2) a2 = i;
    }
    CHECK_NEAR(atoms[a1].r.x(), -3.9184367989026225, 1.0e-12);
    CHECK_NEAR(atoms[a1].r.y(), 2.6440651643797461, 1.0e-12);
    CHECK_NEAR(atoms[a1].r.z(), 5.2690712254285517, 1.0e-12);
    CHECK_NEAR(atoms[a1].v.z(), 5.79013209455442e-04, 1.0e-15);
    CHECK_NEAR(atoms[a1].f.z(), 2.8929546164515996, 1.0e-12);
    CHECK_NEAR(atoms[a1].Ep, -4.0629298955784474, 1.0e-12);
    CHECK_NEAR(atoms[a1].V.trace(), -3.3178872346261723e-01, 1.0e-12);
    CHECK_NEAR(atoms[a2].r.z(), 5.7940689066038047, 1.0e-12);
    CHECK_NEAR(atoms[a2].v.x(), -1.4268458571713898e-03, 1.0e-15);
    CHECK_NEAR(atoms[a2].f.x(), -7.1268568973069453, 1.0e-12);
    CHECK_NEAR(atoms[a2].Ep, -4.2002585997144832, 1.0e-12);
    CHECK_NEAR(atoms[a2].V.trace(), 4.2842826328841377e-01, 1.0e-12);
}

// test/cxx/solver/test_aluminum_bulk_eam.cxx (make_fcc_bulk, md_test_utils.h:291-344)
static void test_aluminum(const std::string& path) {
    const double mass = 26.9815384, a0 = 0.4032;
    tools::Threads threads{1};
    solver::potential::EAM potential{path};
    Atoms atoms;
    const vector basis[4] = {vector(0, 0, 0), vector(0.5, 0.5, 0), vector(0.5, 0, 0.5), vector(0, 0.5, 0.5)};
    const double L = 3 * a0;
    unsigned uid = 1;
    for (int iz = 0; iz < 3; ++iz)
        for (int iy = 0; iy < 3; ++iy)
            for (int ix = 0; ix < 3; ++ix) {
                vector co(-0.5 * L + ix * a0, -0.5 * L + iy * a0, -0.5 * L + iz * a0);
                for (const auto& b : basis) {
                    Atom at{};
                    at.uid = uid++;
                    at.kind = 1;
                    at.m = mass;
                    at.r = co + a0 * b;
                    atoms.push_back(at);
                }
            }
    lattice::Domain domain(-0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L);
    for (int k = 0; k < 3; ++k) domain.set_periodic(k, true);
    set_common(atoms, mass, potential.rcut(), 1.25);
    vector mom = vector::Zero();
    double tm = 0.0;
    for (size_t i = 0; i < atoms.size(); ++i) {
        atoms[i].v << 5e-3 * ((int)(i % 7) - 3), 5e-3 * ((int)((i / 7) % 5) - 2), 5e-3 * ((int)((i / 35) % 3) - 1);
        mom += atoms[i].m * atoms[i].v;
        tm += atoms[i].m;
    }
    for (auto& at : atoms) at.v -= mom / tm;
    solver::boundary::Periodic periodic(domain);
    solver::Single solver(potential, periodic, solver::thermostat::dummy_thermostat, threads);
    solver::stepper::Verlet stepper(solver, threads);
    neibs::VerletList nlist(atoms, atoms, domain, threads);
    CHECK(solver.stages.size() == 2U);
    auto h = run_md_steps(solver, stepper, atoms, nlist, 4e-3, 2, 1);
    CHECK_NEAR(h.back().Etot, -3.4489006959225437e+04, 1.0e-6);
    CHECK_NEAR(h.back().Ep, -6.7190981865001777e+03, 1.0e-6);
    CHECK_NEAR(h.back().Em, -2.7770493824864527e+04, 1.0e-6);
    CHECK_NEAR(h.back().KE, 5.8505213926282473e-01, 1.0e-9);
    CHECK_NEAR(h.back().virial, 7.4272691119381875e+01, 1.0e-9);
    CHECK_NEAR(atoms[0].r.x(), 6.0469801558679681e-01, 1.0e-12);
    CHECK_NEAR(atoms[0].v.x(), -1.3221213313405629e-02, 1.0e-15);
    CHECK_NEAR(atoms[0].f.x(), -1.1358391912725722e+01, 1.0e-12);
    CHECK_NEAR(atoms[0].Ep, -6.3230321656455359e+01, 1.0e-9);
    CHECK_NEAR(atoms[0].Em, -2.5721082474679707e+02, 1.0e-9);
    CHECK_NEAR(atoms[0].V.trace(), 1.3557390418206403e+01, 1.0e-9);
    CHECK(nlist[0].size() > 12U);
}

static Atoms fcc_lattice(int n, double a0, double mass, unsigned seed_kinds) {
    Atoms atoms;
    const vector basis[4] = {vector(0, 0, 0), vector(0.5, 0.5, 0), vector(0.5, 0, 0.5), vector(0, 0.5, 0.5)};
    const double L = n * a0;
    unsigned uid = 1, h = seed_kinds;
    for (int iz = 0; iz < n; ++iz)
        for (int iy = 0; iy < n; ++iy)
            for (int ix = 0; ix < n; ++ix) {
                vector co(-0.5 * L + ix * a0, -0.5 * L + iy * a0, -0.5 * L + iz * a0);
                for (const auto& b : basis) {
                    Atom at{};
                    at.uid = uid++;
                    h = h * 1664525u + 1013904223u;
                    at.kind = seed_kinds ? (unsigned short)((h >> 16) % 5 == 0) : 0;
                    at.m = mass;
                    at.r = co + a0 * b;
                    // a small deterministic displacement so that forces are nonzero
                    at.r += vector(1e-3 * std::sin(1.0 * uid), 1e-3 * std::cos(2.0 * uid), 1e-3 * std::sin(3.0 * uid));
                    atoms.push_back(at);
                }
            }
    return atoms;
}

template <class Solver>
static double total_energy(Solver& solver, Atoms& atoms, neibs::VerletList& nlist) {
    solver.virials(atoms, atoms, nlist.get());
    return measure(atoms).Etot;
}

// problems/NiAl/test-NiAl.py: two EAM kinds, the Ni-Al Pair from its file as
// cross term, Multi with Periodic; then LJs in a Single solver. NVE energy
// must hold, the total force must vanish.
static void test_pair_and_ljs(const std::string& al_path, const std::string& pair_path) {
    const double a0 = 0.405, mass = 26.9815384, dt = 1e-3;
    tools::Threads threads{1};
    solver::potential::EAM al{al_path};
    solver::potential::Pair cross{pair_path};
    CHECK_NEAR(cross.rcut(), 0.6724883999724820, 1e-15);
    for (int form = 0; form < 2; ++form) {
        Atoms atoms = fcc_lattice(5, a0, mass, form == 0 ? 7u : 0u);
        const double L = 5 * a0;
        lattice::Domain domain(-0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L);
        for (int k = 0; k < 3; ++k) domain.set_periodic(k, true);
        solver::boundary::Periodic periodic(domain);
        solver::potential::LJs ljs(0.9, 0.26, 0.62);
        std::unique_ptr<solver::ISolver> solver;
        double rc;
        if (form == 0) {
            auto m = std::make_unique<solver::Multi>(periodic, solver::thermostat::dummy_thermostat, 2, threads);
            m->add_potential(0, 0, al);
            m->add_potential(1, 1, al);
            m->add_potential(0, 1, cross);
            CHECK(m->stages.size() == 2U);
            rc = std::max(al.rcut(), cross.rcut());
            solver = std::move(m);
        } else {
            solver = std::make_unique<solver::Single>(ljs, periodic, solver::thermostat::dummy_thermostat, threads);
            CHECK(solver->stages.size() == 1U);
            rc = ljs.rcut();
        }
        for (auto& at : atoms) {
            at.rcut = rc;
            at.rns = 1.2 * rc;
        }
        solver::stepper::Verlet stepper(*solver, threads);
        neibs::VerletList nlist(atoms, atoms, domain, threads);
        nlist.update(-1.0);
        solver->prepare(atoms, atoms, nlist.get());
        for (auto& st : solver->stages) st(atoms, atoms, nlist.get());
        vector ftot = vector::Zero();
        double fmax = 0.0;
        for (const auto& at : atoms) {
            ftot += at.f;
            fmax = std::max(fmax, at.f.norm());
        }
        CHECK(fmax > 1.0);
        CHECK(ftot.norm() < 1e-9 * fmax * atoms.size());
        const double e0 = total_energy(*solver, atoms, nlist);
        for (int s = 1; s <= 300; ++s) {
            stepper.make_step(atoms, nlist.get(), dt);
            if (nlist.decide()) nlist.update(-1.0);
        }
        const double e1 = total_energy(*solver, atoms, nlist);
        CHECK_NEAR((e1 - e0) / std::fabs(e0), 0.0, 2e-5);
    }
}

// A Langevin thermostat (langevin.cxx:29-42) brings a cold lattice to its
// temperature: <KE> -> 3/2 N kB T over the last steps of the run.
static void test_langevin(const std::string& al_path) {
    const double a0 = 0.4032, mass = 26.9815384, dt = 2e-3, T = 300.0;
    tools::Threads threads{1};
    solver::potential::EAM al{al_path};
    Atoms atoms = fcc_lattice(5, a0, mass, 0u);
    const double L = 5 * a0;
    lattice::Domain domain(-0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L);
    for (int k = 0; k < 3; ++k) domain.set_periodic(k, true);
    solver::boundary::Periodic periodic(domain);
    solver::thermostat::Langevin langevin(5.0, T, dt);
    langevin.set_seed(42);
    solver::thermostat::Compound compound;
    compound.add(langevin);
    solver::Single solver(al, periodic, compound, threads);
    set_common(atoms, mass, al.rcut(), 1.25);
    solver::stepper::Verlet stepper(solver, threads);
    neibs::VerletList nlist(atoms, atoms, domain, threads);
    nlist.update(-1.0);
    double ke = 0.0;
    int samples = 0;
    for (int s = 1; s <= 3000; ++s) {
        stepper.make_step(atoms, nlist.get(), dt);
        if (nlist.decide()) nlist.update(-1.0);
        if (s > 1500 && s % 10 == 0) {
            ke += measure(atoms).KE;
            ++samples;
        }
    }
    const double t_kin = (ke / samples) / (1.5 * atoms.size() * solver::thermostat::Kb);
    std::printf("Langevin: <T_kin> = %.1f K (target %.1f K)\n", t_kin, T);
    CHECK(std::fabs(t_kin - T) < 0.1 * T);
    CHECK_NEAR(langevin.temperature(), T, 0.0);
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::printf("usage: %s <LAMMPS Ar ball> <Al setfl>\n", argv[0]);
        return 2;
    }
    test_verlet_lists();
    test_argon_ball(argv[1]);
    test_aluminum(argv[2]);
    if (argc > 3) test_pair_and_ljs(argv[2], argv[3]);
    test_langevin(argv[2]);
    std::printf("%d checks, %d failures\n", g_checks, g_fail);
    return g_fail == 0 ? 0 : 1;
}
