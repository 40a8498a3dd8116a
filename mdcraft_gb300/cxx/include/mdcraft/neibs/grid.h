// Drop-in header at the path of MDcraft's mdcraft/neibs/grid.h; neibs::Grid is in
// mdcraft/gpu/dropin.h (its build runs on the GPU through mdg_grid_build).
#pragma once
#include <mdcraft/gpu/dropin.h>
