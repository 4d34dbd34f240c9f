// TBB-compatible shim (test infrastructure): forwards to the tbb/ header.
#include "../../tbb/enumerable_thread_specific.h"
