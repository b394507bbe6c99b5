// Oracle build shim: forwards to shim_core.hpp (Xerces-C API subset).
#include "../shim_core.hpp"
