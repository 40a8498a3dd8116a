// mdcraft::data::Atom — the 208-byte atom record of mdcraft/data/atom.h:21-40,
// layout-identical to mdg_atom of the C-ABI so atom vectors cross it without
// conversion.
#pragma once

#include <cstdint>
#include <limits>
#include <vector>

#include <mdcraft/data/vector.h>

#include "mdg.h"

namespace mdcraft {
namespace data {

struct Atom {
    vector r;
    vector v;
    vector f;
    matrix V;
    double m = 0.0;
    double rcut = 0.0;
    double rns = 0.0;
    double Ep = 0.0;
    double Em = 0.0;
    double nc = 0.0;
    unsigned short bc = 0;
    unsigned short kind = 0;
    unsigned int uid = 0;
    unsigned short tag = std::numeric_limits<unsigned short>::max();
};

static_assert(sizeof(Atom) == sizeof(mdg_atom), "Atom must keep MDcraft's 208-byte layout");

using Atoms = std::vector<Atom>;

inline const mdg_atom* as_mdg(const Atoms& a) { return reinterpret_cast<const mdg_atom*>(a.data()); }
inline mdg_atom* as_mdg(Atoms& a) { return reinterpret_cast<mdg_atom*>(a.data()); }

}  // namespace data
}  // namespace mdcraft
