#pragma once
#include <mdcraft/data/vector.h>
