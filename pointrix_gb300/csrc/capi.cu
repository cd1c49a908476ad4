// Library-wide entry points of the C ABI (status names, ABI version).
#include "pgb_common.cuh"

extern "C" {

const char* pgb_status_string(int status) {
  switch (status) {
    case PGB_OK: return "ok";
    case PGB_ERR_INVALID: return "invalid argument";
    case PGB_ERR_CUDA: return "CUDA error";
    case PGB_ERR_OVERFLOW: return "device-side bound exceeded";
    case PGB_ERR_TIMEOUT: return "bounded device wait expired";
    case PGB_ERR_MISMATCH: return "tiles_touched disagrees with uv/radius";
    default: return "unknown status";
  }
}

int pgb_abi_version(void) { return 1; }

}  // extern "C"
