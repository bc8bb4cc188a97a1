// Forwards to the core shim; see core.hpp.
#include "../core.hpp"
