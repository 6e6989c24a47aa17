// Driver-API loader for the reference GPU kernels -- TEST INFRASTRUCTURE ONLY.
//
// Loads oracle/_ref/ref_kernels_bs<N>.cubin (the reference's own kernels,
// compiled from its sources for sm_103a) into the current context and
// launches them with the reference's launch configurations, so golden
// vectors and sm_103a timings of the reference kernels can be recorded.
#include <cuda.h>

#include <cstring>

namespace {
CUmodule g_mod[8] = {};

int ensure_context() {
  CUcontext cur = nullptr;
  if (cuCtxGetCurrent(&cur) != CUDA_SUCCESS) return -1;
  if (cur) return 0;
  CUdevice dev;
  if (cuDeviceGet(&dev, 0) != CUDA_SUCCESS) return -2;
  CUcontext prim;
  if (cuDevicePrimaryCtxRetain(&prim, dev) != CUDA_SUCCESS) return -3;
  return cuCtxSetCurrent(prim) == CUDA_SUCCESS ? 0 : -4;
}
}  // namespace

extern "C" {

int refk_load(int slot, const char* path) {
  if (slot < 0 || slot >= 8) return -10;
  if (cuInit(0) != CUDA_SUCCESS) return -11;
  int rc = ensure_context();
  if (rc) return rc;
  return (int)cuModuleLoad(&g_mod[slot], path);
}

int refk_launch(int slot, const char* name, unsigned gx, unsigned bx, unsigned smem, void* stream,
                void** args) {
  if (slot < 0 || slot >= 8 || !g_mod[slot]) return -10;
  CUfunction f;
  CUresult r = cuModuleGetFunction(&f, g_mod[slot], name);
  if (r != CUDA_SUCCESS) return (int)r;
  if (smem > 48 * 1024) {
    r = cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
    if (r != CUDA_SUCCESS) return (int)r;
  }
  return (int)cuLaunchKernel(f, gx, 1, 1, bx, 1, 1, smem, (CUstream)stream, args, nullptr);
}

}  // extern "C"
