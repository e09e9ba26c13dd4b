// Library-level C-ABI entry points: version, errors, scratch sizing, tableau.
#include <stdio.h>
#include <string.h>

#include "capi_internal.h"
#include "common.cuh"

namespace qg {

static thread_local char g_err[512] = "";

int set_error(int code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return QG_OK;
  snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
  return QG_ERR_CUDA;
}

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cache[dev] == 0) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 148;
    cache[dev] = v;
  }
  return cache[dev];
}

}  // namespace qg

extern "C" int qg_version(void) { return 1; }

extern "C" const char* qg_last_error(void) { return qg::g_err; }

extern "C" int64_t qg_scratch_doubles(void) { return 4096; }

extern "C" int qg_abi_sizes(int64_t* out, int n) {
  const int64_t s[] = {(int64_t)sizeof(qg_csr_groups),   (int64_t)sizeof(qg_dia),
                       (int64_t)sizeof(qg_rk_buffers),   (int64_t)sizeof(qg_state_view),
                       (int64_t)sizeof(qg_batch_system), (int64_t)sizeof(qg_batch_item),
                       (int64_t)sizeof(qg_batch),        (int64_t)sizeof(qg_lindblad),
                       (int64_t)sizeof(qg_dense_lindblad), (int64_t)sizeof(qg_sde)};
  const int m = (int)(sizeof(s) / sizeof(s[0]));
  if (!out) return qg::set_error(QG_ERR_ARG, "null output");
  for (int i = 0; i < m && i < n; ++i) out[i] = s[i];
  return m < n ? m : n;
}

extern "C" int qg_vern7_tableau(double* a, double* b, double* c, double* e, double* bi) {
  using namespace qg;
  if (!a || !b || !c || !e || !bi) return set_error(QG_ERR_ARG, "null output");
  memcpy(a, VERN7_A_HOST, sizeof(double) * 16 * 16);
  memcpy(b, VERN7_B_HOST, sizeof(double) * 10);
  memcpy(c, VERN7_C_HOST, sizeof(double) * 16);
  memcpy(e, VERN7_E_HOST, sizeof(double) * 10);
  memcpy(bi, VERN7_BI_HOST, sizeof(double) * 16 * 7);
  return QG_OK;
}
