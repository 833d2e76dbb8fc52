// Library-level C ABI entry points (version, status strings).
#include "common.cuh"

extern "C" int mgt_abi_version(void) { return 1; }

extern "C" const char* mgt_status_string(int status) {
  switch (status) {
    case MGT_OK: return "ok";
    case MGT_ERR_ARG: return "invalid argument";
    case MGT_ERR_CUDA: return "CUDA runtime error";
    case MGT_ERR_SINGULAR: return "singular matrix (exact zero pivot)";
    case MGT_ERR_TIMEOUT: return "a bounded device-side wait ran out";
    case MGT_ERR_WORKSPACE: return "workspace too small";
    case MGT_ERR_UNSUPPORTED: return "size or mode not supported";
    case MGT_ERR_NOT_CONVERGED: return "iterative refinement did not reach its tolerance";
    default: return "unknown status";
  }
}
