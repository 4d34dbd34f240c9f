// TBB-compatible shim (test infrastructure): forwards to the tbb/ header.
#include "../../tbb/parallel_for.h"
