// TBB-compatible shim (test infrastructure): forwards to the tbb/ header.
#include "../../tbb/concurrent_hash_map.h"
