// Compatibility shim (test infrastructure): included, unused by the simulator.
#pragma once
#include "Vec.h"
