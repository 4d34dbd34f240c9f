// TBB-compatible shim (test infrastructure): forwards to the tbb/ header.
#include "../../tbb/blocked_range2d.h"
