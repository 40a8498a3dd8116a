// MDcraft's C++ neighbour / potential / solver / stepper API as a drop-in
// over libmdg (include/mdg.h).
//
// Class names, constructors and member functions follow the reference:
//   lattice::Domain            mdcraft/lattice/domain.h:77-189
//   tools::Threads             mdcraft/tools/threads.h:28-60   (no-op pool)
//   neibs::ListOne / List      mdcraft/neibs/verlet-list.h:9-123
//   neibs::Grid                mdcraft/neibs/grid.h:14-180
//   neibs::VerletList          mdcraft/neibs/verlet-list.h:134-470
//   solver::potential::Base, LJsCut, LJs, EAM, Pair
//                                          potential/{base,LJs-cut,LJs,EAM,pair}.h
//   solver::boundary::Base, Periodic       boundary/{base,periodic}.h
//   solver::thermostat::Base, Langevin, Compound
//                                          thermostat/{base,langevin,compound}.h
//   solver::ISolver, Single, Multi         solver/{isolver,single,multi}.h
//   solver::stepper::Verlet                solver/stepper/verlet.h
//
// Semantics: the caller keeps owning its `Atoms` vector. Every call uploads
// the atoms to the device system bound to the VerletList, runs the stage on
// the GPU and writes the results back, so host code that reads or edits
// atoms between calls sees the reference's behaviour. For device-resident
// runs use stepper::Verlet::run (the fused driver loop, one transfer each
// way). Errors raise std::runtime_error, like the reference.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <functional>
#include <limits>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include <mdcraft/data/atom.h>

#include "mdg.h"

namespace mdcraft {

namespace gpu {

inline void check(int rc, const char* what) {
    if (rc != MDG_OK) throw std::runtime_error(std::string(what) + ": " + mdg_last_error());
}

// One device context per process (device from MDG_DEVICE, default 0).
inline mdg_ctx* context() {
    static std::unique_ptr<mdg_ctx, int (*)(mdg_ctx*)> ctx(
        [] {
            mdg_ctx* c = nullptr;
            const char* d = std::getenv("MDG_DEVICE");
            check(mdg_ctx_create(d ? std::atoi(d) : 0, &c), "mdg_ctx_create");
            return c;
        }(),
        mdg_ctx_destroy);
    return ctx.get();
}

}  // namespace gpu

// ---------------------------------------------------------------------------
namespace lattice {

class Domain {
public:
    Domain() : Domain(0.0, 1.0, 0.0, 1.0, 0.0, 1.0) {}
    Domain(double xmin, double xmax, double ymin, double ymax, double zmin, double zmax) {
        reshape(xmin, xmax, ymin, ymax, zmin, zmax);
        m_periodic = {false, false, false};
        m_dim = std::fabs(zmin - zmax) > 1e-15 ? 3 : std::fabs(ymin - ymax) > 1e-15 ? 2 : 1;
    }
    void reshape(double xmin, double xmax, double ymin, double ymax, double zmin, double zmax) {
        m_bmin = {xmin, ymin, zmin};
        m_bmax = {xmax, ymax, zmax};
        m_size = {xmax - xmin, ymax - ymin, zmax - zmin};
        m_dim = zmin == zmax ? (ymin == ymax ? 1 : 2) : 3;
    }
    void set_periodic(int axis, bool val) { m_periodic[axis] = val; }
    int dim() const { return m_dim; }
    double xmin() const { return m_bmin[0]; }
    double ymin() const { return m_bmin[1]; }
    double zmin() const { return m_bmin[2]; }
    double xmax() const { return m_bmax[0]; }
    double ymax() const { return m_bmax[1]; }
    double zmax() const { return m_bmax[2]; }
    double xsize() const { return m_size[0]; }
    double ysize() const { return m_size[1]; }
    double zsize() const { return m_size[2]; }
    double bmin(int a) const { return m_bmin[a]; }
    double bmax(int a) const { return m_bmax[a]; }
    double size(int a) const { return m_size[a]; }
    bool periodic(int a) const { return m_periodic[a]; }
    bool xperiodic() const { return m_periodic[0]; }
    bool yperiodic() const { return m_periodic[1]; }
    bool zperiodic() const { return m_periodic[2]; }

    bool belong(data::vector p) const {
        bool in = true;
        for (int i = 0; i < 3; ++i) in = in && (m_bmin[i] <= p[i] && p[i] <= m_bmax[i]);
        return in;
    }
    void fit_in_period(data::vector& v) const {
        for (int i = 0; i < 3; ++i)
            if (m_periodic[i])
                v[i] = v[i] < m_bmin[i] ? v[i] + m_size[i] : v[i] > m_bmax[i] ? v[i] - m_size[i] : v[i];
    }
    data::vector shortest(data::vector v) const {
        for (int i = 0; i < 3; ++i) {
            if (!m_periodic[i]) continue;
            v[i] = std::fabs(v[i] + m_size[i]) < std::fabs(v[i]) ? v[i] + m_size[i] : v[i];
            v[i] = std::fabs(v[i] - m_size[i]) < std::fabs(v[i]) ? v[i] - m_size[i] : v[i];
        }
        return v;
    }
    double nearest_distance(data::vector v, int axis) const {
        double dist = std::numeric_limits<double>::max();
        if (m_periodic[axis])
            dist = std::min(std::fabs(v[axis] - m_bmin[axis]), std::fabs(v[axis] - m_bmax[axis]));
        return dist;
    }
    mdg_domain to_mdg() const {
        mdg_domain d;
        for (int i = 0; i < 3; ++i) {
            d.bmin[i] = m_bmin[i];
            d.bmax[i] = m_bmax[i];
            d.periodic[i] = m_periodic[i] ? 1 : 0;
        }
        return d;
    }

private:
    int m_dim = 3;
    std::array<double, 3> m_bmin{}, m_bmax{}, m_size{};
    std::array<bool, 3> m_periodic{};
};

inline Domain dummy_domain(0.0, 1.0, 0.0, 1.0, 0.0, 1.0);

}  // namespace lattice

// ---------------------------------------------------------------------------
namespace tools {

// The GPU engine does not use host threads; the pool keeps the reference's
// interface (count, on/off, active) for API compatibility.
class Threads {
public:
    explicit Threads(int count = 1000000) { resize(count); }
    void on() { resize(m_max); }
    void off() { resize(1); }
    void resize(int count) { m_count = std::max(1, std::min(count, m_max)); }
    int count() const { return m_count; }
    int max_count() const { return m_max; }
    bool active() const { return m_count > 1; }
    bool disabled() const { return m_count < 2; }

private:
    int m_count = 1;
    int m_max = 1024;
};

inline Threads dummy_pool(1);

}  // namespace tools

// ---------------------------------------------------------------------------
namespace neibs {

using data::Atom;
using data::Atoms;
using data::vector;
using lattice::Domain;
using tools::Threads;
using point_id = std::size_t;

class ListOne : public std::vector<point_id> {
public:
    ListOne() = default;
    explicit ListOne(bool half) : half_(half) {}
    ListOne(std::initializer_list<point_id> init, bool half = false) : std::vector<point_id>(init), half_(half) {}
    bool half() const { return half_; }
    void set_half(bool h) { half_ = h; }

private:
    bool half_ = false;
};

class VerletList;

// The full list; it carries the device system so that solvers and steppers
// handed `nlist.get()` find the atoms' device copy.
class List : public std::vector<ListOne> {
public:
    List() = default;
    explicit List(std::size_t n) : std::vector<ListOne>(n) {}
    VerletList* owner = nullptr;
};

// Grid (grid.h:14-180): build() runs the bounds pass on the GPU
// (mdg_grid_build); the index queries are the reference's integer
// arithmetic on the grid it returns (grid.cxx:107-207).
using cell_id_t = int;
using Index3D = std::array<cell_id_t, 3>;
static constexpr cell_id_t empty_cell = -1;
using Flag3D = std::array<bool, 3>;

struct element_ids {
    cell_id_t cell_id = 0;
    point_id atom_id = 0;
    bool operator<(const element_ids& rhs) const { return cell_id < rhs.cell_id; }
    bool operator==(const element_ids& rhs) const { return cell_id == rhs.cell_id; }
};

class Grid {
public:
    explicit Grid(Domain& domain, Threads& threads = tools::dummy_pool) : domain(domain) {
        (void)threads;
        // Grid::initialize_full (grid.cxx:18-25)
        cell_sizes = {domain.xsize(), domain.ysize(), domain.zsize()};
        domain_num_cells = {1, 1, 1};
        grid_offset = {0, 0, 0};
        num_cells = {1, 1, 1};
    }

    void build(const Atoms& atoms) {
        mdg_domain d = domain.to_mdg();
        mdg_system* sys = nullptr;
        gpu::check(mdg_system_create(gpu::context(), &d, atoms.size(), &sys), "Grid::build");
        int32_t ints[9];
        double dbls[3];
        int rc = atoms.empty() ? MDG_OK : mdg_system_upload_atoms(sys, data::as_mdg(atoms), atoms.size());
        if (rc == MDG_OK) rc = mdg_grid_build(sys, ints, dbls);
        mdg_system_destroy(sys);
        gpu::check(rc, "Grid::build");
        for (int a = 0; a < 3; ++a) {
            domain_num_cells[a] = ints[a];
            grid_offset[a] = ints[3 + a];
            num_cells[a] = ints[6 + a];
            cell_sizes[a] = dbls[a];
        }
    }

    Index3D local_index3D(const vector& v) const {
        Index3D c = global_index3D(v);
        for (int i = 0; i < domain.dim(); ++i) c[i] -= grid_offset[i];
        return c;
    }

    cell_id_t cell_index(const Index3D& ijk) const { return ijk[0] + num_cells[0] * (ijk[1] + num_cells[1] * ijk[2]); }

    void set_indices(Atoms& atoms, std::vector<element_ids>& indices) const {
        indices.resize(atoms.size());
        for (point_id i = 0; i < atoms.size(); ++i) {
            indices[i].cell_id = cell_index(local_index3D(atoms[i].r));
            indices[i].atom_id = i;
        }
    }

    // Grid::adjacent_cells (grid.cxx:138-207)
    std::tuple<std::array<cell_id_t, 27>, Flag3D> adjacent_cells(const vector& r) const {
        const Index3D cell = global_index3D(r);
        std::array<cell_id_t, 27> list;
        int size = 0;
        const bool per[3] = {domain.xperiodic(), domain.yperiodic(), domain.zperiodic()};
        for (cell_id_t x : {-1, 0, 1}) {
            if (per[0] && ((domain_num_cells[0] == 1 && x != 0) || (domain_num_cells[0] == 2 && x == 1))) continue;
            for (cell_id_t y : {-1, 0, 1}) {
                if (per[1] && ((domain_num_cells[1] == 1 && y != 0) || (domain_num_cells[1] == 2 && y == 1)))
                    continue;
                for (cell_id_t z : {-1, 0, 1}) {
                    if (per[2] && ((domain_num_cells[2] == 1 && z != 0) || (domain_num_cells[2] == 2 && z == 1)))
                        continue;
                    Index3D nb = {cell[0] + x, cell[1] + y, cell[2] + z};
                    for (int a = 0; a < 3; ++a) {
                        if (per[a]) nb[a] = (nb[a] + domain_num_cells[a]) % domain_num_cells[a];
                        nb[a] -= grid_offset[a];
                    }
                    if (0 <= nb[0] && nb[0] < num_cells[0] && 0 <= nb[1] && nb[1] < num_cells[1] && 0 <= nb[2] &&
                        nb[2] < num_cells[2])
                        list[size++] = cell_index(nb);
                }
            }
        }
        for (int i = size; i < 27; ++i) list[i] = empty_cell;
        Flag3D is_edge = {false, false, false};
        for (int i = 0; i < domain.dim(); ++i) is_edge[i] = cell[i] == 0 || cell[i] == num_cells[i] - 1;
        return {list, is_edge};
    }

    double cell_size() const { return std::max(cell_sizes[0], std::max(cell_sizes[1], cell_sizes[2])); }
    cell_id_t cells_number() const { return num_cells[0] * num_cells[1] * num_cells[2]; }

private:
    Index3D global_index3D(const vector& v) const {
        Index3D c = {0, 0, 0};
        for (int i = 0; i < domain.dim(); ++i) c[i] = (cell_id_t)std::floor((v[i] - domain.bmin(i)) / cell_sizes[i]);
        return c;
    }

    Domain& domain;
    Index3D domain_num_cells{};
    std::array<double, 3> cell_sizes{};
    Index3D grid_offset{};
    Index3D num_cells{};
};

class VerletList {
public:
    VerletList(Atoms& atoms, Atoms& neibs, Domain& domain, Threads& threads = tools::dummy_pool, bool half = false)
        : m_atoms(&atoms), m_domain(domain), m_half(half) {
        if (&neibs != &atoms && neibs.data() != atoms.data())
            throw std::runtime_error("libmdg drop-in: neighbours must be searched among the same atoms");
        if (m_half && threads.active())
            throw std::runtime_error(
                "Half Verlet lists are currently incompatible with multithreaded pair-force evaluation. "
                "Disable threads or use a full neighbor list.");
        m_list.owner = this;
        m_list.resize(atoms.size());
    }
    VerletList(const VerletList&) = delete;
    VerletList& operator=(const VerletList&) = delete;
    ~VerletList() {
        if (m_sys) mdg_system_destroy(m_sys);
    }

    // VerletList::update (verlet-list.cxx:41-55)
    void update(double kbuf) {
        upload();
        int rc = mdg_nlist_update(m_sys, kbuf, m_half ? 1 : 0);
        if (rc != MDG_OK && rc != MDG_ERR_RANGE) gpu::check(rc, "VerletList::update");
        download();
        refresh_lists();
    }

    // VerletList::decide (verlet-list.cxx:110-158)
    bool decide() const {
        if (!m_sys || m_atoms->size() != m_n) return true;
        const_cast<VerletList*>(this)->upload();
        int need = 1;
        gpu::check(mdg_nlist_decide(m_sys, &need), "VerletList::decide");
        return need != 0;
    }

    List& get() { return m_list; }
    ListOne& operator[](point_id i) { return i < m_list.size() ? m_list[i] : m_dummy; }
    bool is_half() const { return m_half; }
    void set_half(bool b) {
        m_half = b;
        for (auto& l : m_list) l.set_half(b);
    }

    // VerletList::list_for (verlet-list.cxx:251-276)
    ListOne list_for(vector x) const {
        if (!m_sys) return ListOne();
        std::vector<uint64_t> out(65536);
        size_t cnt = 0;
        gpu::check(mdg_nlist_list_for(m_sys, x.data(), out.data(), out.size(), &cnt), "VerletList::list_for");
        ListOne r;
        for (size_t k = 0; k < std::min(cnt, out.size()); ++k) r.push_back(out[k]);
        return r;
    }

    // VerletList::sort (verlet-list.cxx:237-249): wraps `atoms` into the
    // period in place and returns them ordered by owning cell (x fastest),
    // ascending index inside a cell; this list is not changed.
    Atoms sort(Atoms& atoms) {
        Atoms sorted(atoms.size());
        if (atoms.empty()) return sorted;
        if (!m_sys) upload();  // the device system gives the device and the domain
        int rc = mdg_nlist_sort(m_sys, data::as_mdg(atoms), atoms.size(), data::as_mdg(sorted));
        if (rc != MDG_OK && rc != MDG_ERR_RANGE) gpu::check(rc, "VerletList::sort");
        return sorted;
    }

    // Device system of these atoms (uploading the host copy first).
    mdg_system* sync_up() {
        upload();
        return m_sys;
    }
    void sync_down() { download(); }
    // after device-side rebuilds: atoms and lists back to the host
    void sync_down_all() {
        download();
        refresh_lists();
    }
    mdg_system* system() const { return m_sys; }
    Domain& domain() { return m_domain; }

private:
    void upload() {
        if (!m_sys || m_n != m_atoms->size()) {
            if (m_sys) mdg_system_destroy(m_sys);
            m_sys = nullptr;
            mdg_domain d = m_domain.to_mdg();
            gpu::check(mdg_system_create(gpu::context(), &d, m_atoms->size(), &m_sys), "mdg_system_create");
            m_n = m_atoms->size();
        }
        gpu::check(mdg_system_upload_atoms(m_sys, data::as_mdg(*m_atoms), m_n), "upload atoms");
    }
    void download() { gpu::check(mdg_system_download_atoms(m_sys, data::as_mdg(*m_atoms), m_n), "download atoms"); }
    void refresh_lists() {
        size_t tot = 0;
        gpu::check(mdg_nlist_total(m_sys, &tot), "nlist total");
        std::vector<uint64_t> off(m_n + 1), idx(std::max<size_t>(tot, 1));
        gpu::check(mdg_nlist_export(m_sys, off.data(), idx.data(), idx.size()), "nlist export");
        m_list.resize(m_n);
        for (size_t i = 0; i < m_n; ++i) {
            ListOne& l = m_list[i];
            l.clear();
            l.set_half(m_half);
            l.insert(l.end(), idx.begin() + off[i], idx.begin() + off[i + 1]);
        }
    }

    Atoms* m_atoms;
    Domain& m_domain;
    bool m_half;
    List m_list;
    ListOne m_dummy;
    mdg_system* m_sys = nullptr;
    size_t m_n = 0;
};

}  // namespace neibs

// ---------------------------------------------------------------------------
namespace solver {

using data::Atoms;
using NeibsList = neibs::List;
using NeibsListOne = neibs::ListOne;

namespace potential {

enum type : unsigned short { undefined, pair, eam, mtpr, ternary };

class Base {
public:
    Base(double rcut, unsigned short t) : type(t), m_rcut(rcut) {}
    virtual ~Base() {
        if (m_pot) mdg_pot_destroy(m_pot);
    }
    double rcut() { return m_rcut; }
    mdg_potential* handle() const { return m_pot; }
    const unsigned short type;

    // Potential::value over arrays of squared distances (base.h:41-42; the
    // pair energy term, EAM.cxx:141-174, pair.cxx:81-114, LJs.cxx:61-71;
    // 0 for LJsCut, base.cxx:19), evaluated on the GPU
    void value(const double* r2, double* Uout, std::size_t size) {
        gpu::check(mdg_pot_values(gpu::context(), m_pot, r2, size, Uout), "Potential::value");
    }
    double value(const double* r2, std::size_t size) {
        std::vector<double> u(size);
        value(r2, u.data(), size);
        double s = 0.0;
        for (double x : u) s += x;
        return s;
    }

    // The per-atom overloads (base.h:44-56): force, virial and density of
    // one atom over an explicit list of indices into `neibs`, in the list's
    // order with the reference's FP64 arithmetic, on the GPU
    // (mdg_pot_atom; LJsCut: LJs-cut.cxx:22-131, EAM: EAM.cxx:306-354,
    // 465-497, 541-560).
    virtual void force(Atoms::iterator atom, Atoms& neibs, NeibsListOne& nlist) {
        per_atom(MDG_ATOM_FORCE, atom, neibs, nlist);
    }
    virtual void virial(Atoms::iterator atom, Atoms& neibs, NeibsListOne& nlist) {
        per_atom(MDG_ATOM_VIRIAL, atom, neibs, nlist);
    }
    virtual void density(Atoms::iterator atom, Atoms& neibs, NeibsListOne& nlist) {
        per_atom(MDG_ATOM_DENSITY, atom, neibs, nlist);
    }

protected:
    void per_atom(int what, Atoms::iterator atom, Atoms& neibs, NeibsListOne& nlist) {
        if (nlist.empty()) return;
        std::vector<uint64_t> idx(nlist.begin(), nlist.end());
        const int rc = mdg_pot_atom(gpu::context(), m_pot, what, reinterpret_cast<mdg_atom*>(&*atom),
                                    data::as_mdg(neibs), neibs.size(), idx.data(), idx.size(), nlist.half() ? 1 : 0);
        // a density outside the embedding table keeps the reference's
        // extrapolated value, as the reference does
        if (rc != MDG_OK && rc != MDG_ERR_RANGE) gpu::check(rc, "Potential per-atom call");
    }

    double m_rcut;
    mdg_potential* m_pot = nullptr;
};

// LJsCut(a, s, rcut) (LJs-cut.h:15-19)
class LJsCut : public Base {
public:
    LJsCut(double a, double s, double rcut) : Base(rcut, type::pair) {
        gpu::check(mdg_pot_ljcut_create(a, s, rcut, &m_pot), "LJsCut");
    }
};

// EAM(rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh) / EAM(filename) (EAM.h:13-22)
class EAM : public Base {
public:
    EAM(double rcut, const double* Femb, const double* Rho, const double* Vpar, int Nr1, const double dr, int Nrh1,
        const double drh)
        : Base(rcut, type::eam) {
        gpu::check(mdg_pot_eam_create(rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh, &m_pot), "EAM");
    }
    explicit EAM(std::string filename) : Base(0.0, type::eam) {
        gpu::check(mdg_pot_eam_create_from_file(filename.c_str(), &m_pot), "EAM(file)");
        gpu::check(mdg_pot_rcut(m_pot, &m_rcut), "EAM rcut");
    }
    // EAM::embeddingEnergy (EAM.cxx:562-601) on the GPU
    void embeddingEnergy(const double* nr, double* EF, double* dF, std::size_t size) {
        gpu::check(mdg_pot_embedding(gpu::context(), m_pot, nr, size, EF, dF), "EAM::embeddingEnergy");
    }
};

// LJs(aVr, rVr, Rcutoff) (LJs.h:14-18)
class LJs : public Base {
public:
    LJs(double aVr, double rVr, double Rcutoff) : Base(Rcutoff, type::pair) {
        gpu::check(mdg_pot_ljs_create(aVr, rVr, Rcutoff, &m_pot), "LJs");
    }
};

// Pair(Rcutoff, Vpar, Nr1, dr) / Pair(filename) (pair.h:13-18)
class Pair : public Base {
public:
    Pair(double Rcutoff, const double* Vpar, int Nr1, const double dr) : Base(Rcutoff, type::pair) {
        gpu::check(mdg_pot_pair_create(Rcutoff, Vpar, Nr1, dr, &m_pot), "Pair");
    }
    explicit Pair(std::string filename) : Base(0.0, type::pair) {
        gpu::check(mdg_pot_pair_create_from_file(filename.c_str(), &m_pot), "Pair(file)");
        gpu::check(mdg_pot_rcut(m_pot, &m_rcut), "Pair rcut");
    }
};

}  // namespace potential

namespace boundary {
class Base {
public:
    explicit Base(lattice::Domain& domain = lattice::dummy_domain) : m_domain(domain) {}
    virtual ~Base() = default;
    virtual bool periodic() const { return false; }
    lattice::Domain& get_domain() { return m_domain; }

protected:
    lattice::Domain& m_domain;
};
inline Base dummy_boundary;

// boundary::Periodic(Domain&) (periodic.h:29): ghost images across periodic
// faces, evaluated inside the force kernels.
class Periodic : public Base {
public:
    explicit Periodic(lattice::Domain& domain) : Base(domain) {}
    bool periodic() const override { return true; }
};
}  // namespace boundary

namespace thermostat {
const double Kb = 0.008314462175;
// thermostat::Base (thermostat/base.h): applies nothing.
class Base {
public:
    virtual ~Base() {
        if (m_t) mdg_thermo_destroy(m_t);
    }
    mdg_thermostat* handle() const { return m_t; }

protected:
    mdg_thermostat* m_t = nullptr;
};
inline Base dummy_thermostat;

// Langevin(beta, temperature, time_step, heat_x, heat_y, heat_z, Ux, Uy, Uz,
// xmin, xmax) (langevin.h:17-29). Like the reference it seeds its random
// stream from std::random_device; set_seed makes a run repeatable.
class Langevin : public Base {
public:
    Langevin(double beta, double temperature, double time_step, int heat_x = 1, int heat_y = 1, int heat_z = 1,
             double Ux = 0.0, double Uy = 0.0, double Uz = 0.0, double xmin = -1e+15, double xmax = 1e+15) {
        m_p.beta = beta;
        m_p.temperature = temperature;
        m_p.time_step = time_step;
        m_p.heat[0] = heat_x;
        m_p.heat[1] = heat_y;
        m_p.heat[2] = heat_z;
        m_p.U[0] = Ux;
        m_p.U[1] = Uy;
        m_p.U[2] = Uz;
        m_p.xmin = xmin;
        m_p.xmax = xmax;
        std::random_device rd;
        m_p.seed = ((uint64_t)rd() << 32) ^ (uint64_t)rd();
        gpu::check(mdg_thermo_langevin_create(&m_p, &m_t), "Langevin");
    }
    void set_friction(double beta) {
        m_p.beta = beta;
        push();
    }
    void set_temperature(double T) {
        m_p.temperature = T;
        push();
    }
    void set_average_velocity(data::vector U) {
        for (int k = 0; k < 3; ++k) m_p.U[k] = U[k];
        push();
    }
    void set_heating_axes(int heat_x = 1, int heat_y = 1, int heat_z = 1) {
        m_p.heat[0] = heat_x;
        m_p.heat[1] = heat_y;
        m_p.heat[2] = heat_z;
        push();
    }
    void set_dimensions(double xmin, double xmax) {
        m_p.xmin = xmin;
        m_p.xmax = xmax;
        push();
    }
    // GPU-specific: the Philox key of the random force
    void set_seed(uint64_t seed) {
        m_p.seed = seed;
        push();
    }
    double friction() { return m_p.beta; }
    double temperature() { return m_p.temperature; }
    data::vector average_velocity() { return data::vector(m_p.U[0], m_p.U[1], m_p.U[2]); }
    double xmin() { return m_p.xmin; }
    double xmax() { return m_p.xmax; }

private:
    void push() { gpu::check(mdg_thermo_langevin_set(m_t, &m_p), "Langevin set"); }
    mdg_langevin m_p{};
};

// Compound (thermostat/compound.h:12-24): its parts in the order added.
class Compound : public Base {
public:
    Compound() { gpu::check(mdg_thermo_compound_create(&m_t), "Compound"); }
    void add(Base& thermostat) {
        if (thermostat.handle()) gpu::check(mdg_thermo_compound_add(m_t, thermostat.handle()), "Compound add");
    }
};
}  // namespace thermostat

using Potential = potential::Base;
using Boundary = boundary::Base;
using Thermostat = thermostat::Base;
using StageFunc = std::function<void(Atoms&, Atoms&, NeibsList&)>;

inline mdg_system* system_of(NeibsList& nlist) {
    if (!nlist.owner) throw std::runtime_error("libmdg drop-in: the list does not come from a VerletList");
    return nlist.owner->sync_up();
}

class ISolver {
public:
    virtual ~ISolver() {
        if (m_s) mdg_solver_destroy(m_s);
    }
    // Pair::prepare (pair.cxx:16-29). The reference's prepare reads no list,
    // so a list no VerletList owns is accepted: the atoms are then prepared
    // on a device system of their own over the boundary's domain.
    virtual void prepare(Atoms& atoms, Atoms& neibs, NeibsList& nlist) {
        (void)neibs;
        if (nlist.owner) {
            call(mdg_solver_prepare, nlist);
            return;
        }
        mdg_domain d = m_domain->to_mdg();
        mdg_system* sys = nullptr;
        gpu::check(mdg_system_create(gpu::context(), &d, atoms.size(), &sys), "prepare");
        int rc = atoms.empty() ? MDG_OK : mdg_system_upload_atoms(sys, data::as_mdg(atoms), atoms.size());
        if (rc == MDG_OK) rc = mdg_solver_prepare(m_s, sys);
        if (rc == MDG_OK && !atoms.empty()) rc = mdg_system_download_atoms(sys, data::as_mdg(atoms), atoms.size());
        mdg_system_destroy(sys);
        gpu::check(rc, "prepare");
    }
    void charge(Atoms&, Atoms&, NeibsList& nlist) { call(mdg_solver_charge, nlist); }
    void forces(Atoms&, Atoms&, NeibsList& nlist) { call(mdg_solver_forces, nlist); }
    void virials(Atoms&, Atoms&, NeibsList& nlist) { call(mdg_solver_virials, nlist); }
    // GPU-specific: FP64 reference arithmetic (default) or mixed precision
    void set_precision(int p) { gpu::check(mdg_solver_set_precision(m_s, p), "set_precision"); }
    mdg_solver* handle() const { return m_s; }

    std::vector<StageFunc> stages;

protected:
    void call(int (*fn)(mdg_solver*, mdg_system*), NeibsList& nlist) {
        mdg_system* sys = system_of(nlist);
        gpu::check(fn(m_s, sys), "solver stage");
        nlist.owner->sync_down();
    }
    void make_stages() {
        int n = 0;
        gpu::check(mdg_solver_num_stages(m_s, &n), "num_stages");
        stages.clear();
        if (n == 2)
            stages.emplace_back([this](Atoms& a, Atoms& b, NeibsList& l) { charge(a, b, l); });
        if (n >= 1)
            stages.emplace_back([this](Atoms& a, Atoms& b, NeibsList& l) { forces(a, b, l); });
    }
    mdg_solver* m_s = nullptr;
    lattice::Domain* m_domain = &lattice::dummy_domain;  // the boundary's domain
};

using Pair = ISolver;

// Single(pot, boundary, thermostat, threads) (single.h:37-42)
class Single : public ISolver {
public:
    Single(Potential& potential, Boundary& boundary = boundary::dummy_boundary,
           Thermostat& thermostat = thermostat::dummy_thermostat, tools::Threads& threads = tools::dummy_pool) {
        (void)threads;
        m_domain = &boundary.get_domain();
        gpu::check(mdg_solver_single(potential.handle(), boundary.periodic() ? 1 : 0, &m_s), "Single");
        if (thermostat.handle()) gpu::check(mdg_solver_set_thermostat(m_s, thermostat.handle()), "thermostat");
        make_stages();
    }
};

// Multi(boundary, thermostat, nkinds, threads) + add_potential (multi.h:42-49)
class Multi : public ISolver {
public:
    Multi(Boundary& boundary = boundary::dummy_boundary, Thermostat& thermostat = thermostat::dummy_thermostat,
          std::size_t nkinds = 1, tools::Threads& threads = tools::dummy_pool) {
        (void)threads;
        m_domain = &boundary.get_domain();
        gpu::check(mdg_solver_multi((int)nkinds, boundary.periodic() ? 1 : 0, &m_s), "Multi");
        if (thermostat.handle()) gpu::check(mdg_solver_set_thermostat(m_s, thermostat.handle()), "thermostat");
    }
    void add_potential(std::size_t i, std::size_t j, Potential& pot) {
        gpu::check(mdg_solver_add_potential(m_s, (int)i, (int)j, pot.handle()), "add_potential");
        make_stages();
    }
};

namespace stepper {

// stepper::Verlet(solver, threads) (verlet.h:34-64)
class Verlet {
public:
    explicit Verlet(ISolver& solver, tools::Threads& threads = tools::dummy_pool) : m_solver(solver) {
        (void)threads;
    }
    // Verlet::make_step (verlet.cxx:36-48)
    void make_step(Atoms& atoms, NeibsList& nlist, double dt) {
        (void)atoms;
        mdg_system* sys = system_of(nlist);
        gpu::check(mdg_verlet_make_step(m_solver.handle(), sys, dt), "make_step");
        nlist.owner->sync_down();
    }
    // The driver loop {make_step; if decide(): update(-1)} x steps, device
    // resident between the two transfers.
    void run(Atoms& atoms, NeibsList& nlist, double dt, long steps) {
        (void)atoms;
        mdg_system* sys = system_of(nlist);
        int rc = mdg_run(m_solver.handle(), sys, dt, steps);
        if (rc != MDG_OK && rc != MDG_ERR_RANGE) gpu::check(rc, "run");
        nlist.owner->sync_down_all();
    }

private:
    ISolver& m_solver;
};

}  // namespace stepper
}  // namespace solver
}  // namespace mdcraft
