// Drop-in header at the path of MDcraft's mdcraft/solver/potential/LJs.h; the classes are in
// mdcraft/gpu/dropin.h (libmdg C-ABI underneath).
#pragma once
#include <mdcraft/gpu/dropin.h>
