// Kernel k-means (popcorn formulation): kernel-matrix build and iteration.
#include "km_lloyd.cuh"

struct km_kkm {
  km_kkm_params p;
};

extern "C" {

km_status km_kernel_matrix(const float*, uint64_t, uint32_t, int32_t, float, float, int32_t, float,
                           int32_t, int32_t, void*, float*, void*) {
  return KM_ERR_UNSUPPORTED;
}

km_status km_kkm_create(const km_kkm_params* p, km_kkm** out) {
  if (!p || !out) return KM_ERR_ARG;
  *out = nullptr;
  return KM_ERR_UNSUPPORTED;
}

km_status km_kkm_set_data(km_kkm* h, const float* X, int) {
  if (!h || !X) return KM_ERR_ARG;
  return KM_ERR_UNSUPPORTED;
}

km_status km_kkm_fit(km_kkm* h, const uint32_t*, uint32_t*, km_result*) {
  if (!h) return KM_ERR_ARG;
  return KM_ERR_UNSUPPORTED;
}

void km_kkm_destroy(km_kkm* h) { delete h; }

}  // extern "C"
