// Compatibility shim (test infrastructure): included, unused by the compiled
// paths of the simulator.
#pragma once
#include "vec2.h"
