// Error reporting for the C ABI: a per-thread message buffer read back with
// lbm_last_error(); every entry point returns an int status.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "lbm_common.cuh"

namespace {
thread_local char g_msg[512] = "";
}

namespace lbm_err {

int set(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  return code;
}

int cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return LBM_OK;
  return set(LBM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int launch(const char* what) { return cuda(cudaGetLastError(), what); }

}  // namespace lbm_err

extern "C" {

int lbm_abi_version(void) { return LBM_GB300_ABI_VERSION; }

int lbm_last_error(char* buf, int64_t buflen) {
  if (!buf || buflen <= 0) return LBM_ERR_ARG;
  std::strncpy(buf, g_msg, (size_t)buflen - 1);
  buf[buflen - 1] = '\0';
  return LBM_OK;
}

}  // extern "C"
