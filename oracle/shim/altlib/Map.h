// Compatibility shim (test infrastructure): the simulator includes this
// header but uses nothing from it.
#pragma once
