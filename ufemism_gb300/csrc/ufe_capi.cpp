// C-ABI glue: error reporting, device probe, host mesh substrate entry point.
#include <cstdio>
#include <cstring>
#include <string>

#include "ufe_internal.h"

namespace ufe {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return UFE_OK;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return UFE_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return UFE_NO_DEVICE;
  return UFE_CUDA_ERROR;
}

}  // namespace ufe

using namespace ufe;

extern "C" const char *ufe_last_error_string(void) { return g_last_error.c_str(); }

extern "C" int ufe_init(int device) {
  int n = 0;
  int rc = cuda_status(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
  if (rc) return UFE_NO_DEVICE;
  if (device < 0 || device >= n) { set_error("ufe_init: no such device"); return UFE_NO_DEVICE; }
  rc = cuda_status(cudaSetDevice(device), "cudaSetDevice");
  if (rc) return UFE_NO_DEVICE;
  cudaDeviceProp prop;
  rc = cuda_status(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  if (rc) return UFE_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "ufe_init: device is sm_%d%d; this library is built for sm_103a only",
                  prop.major, prop.minor);
    set_error(buf);
    return UFE_NO_DEVICE;
  }
  if (!prop.cooperativeLaunch) { set_error("ufe_init: device lacks cooperative launch"); return UFE_NO_DEVICE; }
  return UFE_OK;
}

extern "C" int ufe_aaac_build(const ufe_base_mesh *base, ufe_aaac_mesh *out) {
  if (!base || !out || !base->V || !base->nC || !base->C || !base->niTri || !base->iTri || !base->Tri ||
      !base->edge_index || !out->iAci || !out->Aci || !out->edge_index_Ac || !out->nCAaAc || !out->CAaAc ||
      !out->Nx_AaAc || !out->Ny_AaAc || !out->Nxx_AaAc || !out->Nxy_AaAc || !out->Nyy_AaAc ||
      (out->colour && (!out->colour_vi || !out->colour_nV))) {
    set_error("ufe_aaac_build: missing array");
    return UFE_BAD_ARG;
  }
  std::string msg;
  const int rc = aaac_build(base, out, &msg);
  if (rc) set_error("ufe_aaac_build: " + msg);
  return rc;
}
