// Lloyd engine host code: buffers, preparation and the per-iteration launch
// sequence (assign -> refine -> sort -> update -> finalize -> control).
#include "km_lloyd.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

namespace km {

namespace {
thread_local std::string g_last_error;

template <class T>
km_status dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    set_last_error(e, "cudaMalloc", __FILE__, __LINE__);
    (void)cudaGetLastError();
    return KM_ERR_ALLOC;
  }
  return KM_OK;
}

template <class T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

uint32_t round_up(uint32_t v, uint32_t m) { return (v + m - 1) / m * m; }
}  // namespace

void set_last_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
}

const char* last_error_text() { return g_last_error.c_str(); }

// Relative error coefficients of the fast distance path (see TieBound).
TieBound make_tie_bound(int precision, uint32_t d, bool a_exact) {
  const double u = std::ldexp(1.0, -24);
  const double ub = std::ldexp(1.0, -8);
  const double uacc = std::ldexp(1.0, -22);  // tensor-core FP32 accumulation, 4 ulp per add
  auto gamma = [](double m, double uu) { return m * uu / (1.0 - m * uu); };
  double eps;
  if (precision == KM_PREC_FP32) {
    eps = gamma((double)d, u);
  } else if (precision == KM_PREC_BF16) {
    // |x^ c^ - x c| <= (2ub + ub^2) |x||c| per term (ub only when x^ = x),
    // plus FP32 accumulation of d products
    eps = a_exact ? ub + (1 + ub) * gamma((double)d, uacc)
                  : 2 * ub + ub * ub + (1 + ub) * (1 + ub) * gamma((double)d, uacc);
  } else if (a_exact) {
    // split-2: c = c_hi + c_lo + r, |r| <= ub^2 |c|; 2d exact products accumulated
    eps = ub * ub + (1 + 2 * ub) * gamma(2.0 * d, uacc);
  } else {
    eps = 3.5 * ub * ub + (1 + 5 * ub) * gamma(3.0 * d, uacc);
  }
  TieBound tb;
  tb.A = (float)(2.02 * eps + 2.1 * u);
  tb.B = (float)(2.1 * u);
  tb.g = (float)(gamma((double)d + 2.0, u) * 1.01);
  tb.safety = 1.25f;
  return tb;
}

LloydEngine::~LloydEngine() {
  if (device >= 0) cudaSetDevice(device);
  dfree(X_owned); dfree(xn2); dfree(xn2d); dfree(Xb); dfree(Xlo);
  dfree(C); dfree(Cn); dfree(cn2); dfree(dsq); dfree(objpart); dfree(shift_c); dfree(obj_c);
  dfree(Cb); dfree(Clo); dfree(labels); dfree(mindist); dfree(queue); dfree(qfull); dfree(Ct);
  dfree(qcnt); dfree(qfcnt); dfree(qwide); dfree(qwcnt); dfree(wlc); dfree(wl);
  dfree(q2); dfree(q2full); dfree(q2cnt); dfree(q2fcnt); dfree(fidx); dfree(nfull);
  dfree(seghist); dfree(counts); dfree(cstart); dfree(order); dfree(perm); dfree(red_part); dfree(st);
  if (h_st) cudaFreeHost(h_st);
  for (auto& l : kmat_lists)
    if (l.dev) cudaFree(l.dev);
  if (aux) cudaStreamDestroy(aux);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

km_status LloydEngine::init(uint64_t n_, uint32_t d_, uint32_t k_, int precision_, int device_,
                            void* stream_, bool need_update) {
  if (n_ == 0 || d_ == 0 || k_ == 0 || k_ > n_) return KM_ERR_ARG;
  if (n_ >= (1ull << 32) - 256) return KM_ERR_ARG;           // labels / perm are 32-bit
  if ((uint64_t)d_ * n_ / d_ != n_) return KM_ERR_ARG;
  if (precision_ < KM_PREC_FP32 || precision_ > KM_PREC_BF16X3) return KM_ERR_ARG;
  n = n_; d = d_; k = k_; precision = precision_; device = device_;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { (void)cudaGetLastError(); return KM_ERR_NO_DEVICE; }
  if (device < 0 || device >= ndev) return KM_ERR_ARG;
  KM_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  KM_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3) return KM_ERR_NO_DEVICE;  // code is built for sm_103a only
  num_sms = prop.multiProcessorCount;
  if (stream_) {
    stream = static_cast<cudaStream_t>(stream_);
  } else {
    KM_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
  }
  dp = round_up(d, 64);
  kp = round_up(std::max<uint32_t>(k, 16), 16);
  if (precision != KM_PREC_FP32) {
    // planned for the widest operands of the precision; SPLIT2 (chosen at
    // set_points when the points turn out to be exact BF16) needs less
    const int plan_mode = precision == KM_PREC_BF16X3 ? TC_SPLIT3 : TC_PLAIN;
    if (kp <= 256) tc = plan_tc(dp, kp, plan_mode, n, num_sms);
    if (!tc.ok) {
      // k > 256, or the centroid operand does not fit shared memory whole
      tc = plan_tc_chunked(dp, k, plan_mode, n, num_sms);
      if (tc.ok) kp = tc.kp;            // centroid operand padded to whole chunks
    }
    if (!tc.ok) return KM_ERR_UNSUPPORTED;
    KM_TRY(tc_set_attributes(tc, plan_mode));
    if (plan_mode == TC_SPLIT3) KM_TRY(tc_set_attributes(tc, TC_SPLIT2));
    tc_mode = plan_mode;
  }
  tb = make_tie_bound(precision, d, false);

  KM_TRY(dalloc(&xn2, n));
  KM_TRY(dalloc(&xn2d, n));
  if (precision != KM_PREC_FP32) {
    KM_TRY(dalloc(&Xb, (size_t)n * dp));
    KM_TRY(dalloc(&Cb, (size_t)kp * dp));
    if (precision == KM_PREC_BF16X3) {
      KM_TRY(dalloc(&Xlo, (size_t)n * dp));
      KM_TRY(dalloc(&Clo, (size_t)kp * dp));
    }
  }
  KM_TRY(dalloc(&C, (size_t)k * d));
  KM_TRY(dalloc(&cn2, (kp + 63) & ~63u));        // padded: +inf up to a multiple of 64
  KM_TRY(dalloc(&labels, n));
  KM_TRY(dalloc(&mindist, n));
  {
    const uint64_t rows = (n + 127) / 128 * 128;     // whole 128-row tiles
    KM_TRY(dalloc(&queue, rows));
    KM_TRY(dalloc(&qfull, rows));
    KM_TRY(dalloc(&qcnt, rows / 32));
    KM_TRY(dalloc(&qfcnt, rows / 32));
    rq = RefineQueues{queue, qfull, qcnt, qfcnt, rows / 32};
    if (precision != KM_PREC_FP32 && tc.chunked) {
      // candidate lists of the chunked distance kernel: up to 256 per row,
      // fewer when the lists would pass 16 GiB
      uint32_t L = 256;
      while (L > 32 && (uint64_t)rows * L * sizeof(uint2) > (16ull << 30)) L -= 32;
      KM_TRY(dalloc(&qwide, rows));
      KM_TRY(dalloc(&qwcnt, rows / 32));
      KM_TRY(dalloc(&wlc, rows));
      KM_TRY(dalloc(&wl, (size_t)rows * L));
      rq.wide = qwide; rq.wcnt = qwcnt; rq.wl = wl; rq.wlc = wlc; rq.L = L;
      KM_TRY(dalloc(&q2, rows));
      KM_TRY(dalloc(&q2full, rows));
      KM_TRY(dalloc(&q2cnt, rows / 32));
      KM_TRY(dalloc(&q2fcnt, rows / 32));
      KM_TRY(dalloc(&fidx, rows));
      KM_TRY(dalloc(&nfull, 1));
      rq2 = RefineQueues{q2, q2full, q2cnt, q2fcnt, rows / 32};
      tb32 = make_tie_bound(KM_PREC_FP32, d, false);
    }
  }
  KM_TRY(dalloc(&Ct, (size_t)k * d));
  KM_TRY(dalloc(&red_part, 256));
  KM_TRY(dalloc(&st, 1));
  KM_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&h_st), sizeof(DevState)));
  std::memset(h_st, 0, sizeof(DevState));
  KM_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(DevState), stream));

  // Stable-sort geometry: segments of `seg` rows, k x nseg counts.
  seg = 1024;
  nseg = (uint32_t)((n + seg - 1) / seg);
  while ((uint64_t)k * nseg > (16ull << 20) && seg < (1u << 30)) {
    seg <<= 1;
    nseg = (uint32_t)((n + seg - 1) / seg);
  }
  const size_t per_warp = (size_t)k * 4;
  if (per_warp <= 6144) sort_wpb = 8;
  else sort_wpb = (int)std::max<size_t>(1, (48 * 1024) / per_warp);
  sort_smem = per_warp * sort_wpb;
  if (sort_smem > 227 * 1024) return KM_ERR_UNSUPPORTED;
  if (sort_smem > 48 * 1024) {
    KM_CUDA_TRY(cudaFuncSetAttribute(seg_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem));
    KM_CUDA_TRY(cudaFuncSetAttribute(seg_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem));
  }
  KM_TRY(refine_prepare());
  if (need_update) {
    KM_TRY(update_sums_prepare());
    KM_TRY(dalloc(&Cn, (size_t)k * d));
    KM_TRY(dalloc(&dsq, (size_t)k * d));
    KM_TRY(dalloc(&objpart, (size_t)k * d));
    KM_TRY(dalloc(&shift_c, k));
    KM_TRY(dalloc(&obj_c, k));
    KM_TRY(dalloc(&seghist, (size_t)k * nseg));
    KM_TRY(dalloc(&counts, k));
    KM_TRY(dalloc(&cstart, (size_t)k + 1));
    KM_TRY(dalloc(&order, k));
    KM_TRY(dalloc(&perm, n));
  }
  return KM_OK;
}

km_status LloydEngine::set_points(const float* Xsrc, bool on_device, bool copy) {
  KM_CUDA_TRY(cudaSetDevice(device));
  const size_t bytes = sizeof(float) * n * d;
  // A large host source is copied in row chunks alternating between the
  // handle's stream and a second one (two copy engines), and each chunk's
  // preparation (norms, BF16 copies) runs behind its own copy, overlapping
  // the copies of the chunks after it.
  const bool chunked = !on_device && bytes >= (64ull << 20);
  if (copy || !on_device) {
    if (!X_owned) KM_TRY(dalloc(&X_owned, (size_t)n * d));
    X = X_owned;
  } else {
    X = Xsrc;
  }
  refine_v4 = (d % 4 == 0) && (reinterpret_cast<uintptr_t>(X) % 16 == 0);
  KM_CUDA_TRY(cudaMemsetAsync(&st->err, 0, sizeof(uint32_t), stream));
  KM_CUDA_TRY(cudaMemsetAsync(&st->x_not_bf16, 0, sizeof(uint32_t), stream));
  if (chunked) {
    if (!aux) {
      KM_CUDA_TRY(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
      KM_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      KM_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
    KM_CUDA_TRY(cudaEventRecord(ev_fork, stream));
    KM_CUDA_TRY(cudaStreamWaitEvent(aux, ev_fork, 0));
    const uint64_t nch = 8, rows = (n + nch - 1) / nch;
    for (uint64_t c = 0; c < nch; ++c) {
      const uint64_t r0 = c * rows, r1 = std::min<uint64_t>(n, r0 + rows);
      if (r0 >= r1) break;
      cudaStream_t sc = (c & 1) ? aux : stream;
      KM_CUDA_TRY(cudaMemcpyAsync(X_owned + r0 * d, Xsrc + r0 * d, sizeof(float) * (r1 - r0) * d,
                                  cudaMemcpyHostToDevice, sc));
      const int blocks = (int)std::min<uint64_t>((r1 - r0 + 7) / 8, (uint64_t)num_sms * 8);
      prep_points_kernel<<<blocks, 256, 0, sc>>>(X + r0 * d, r1 - r0, d, dp, xn2 + r0, xn2d + r0,
                                                 Xb ? Xb + r0 * dp : nullptr, Xlo ? Xlo + r0 * dp : nullptr, st);
    }
    KM_CUDA_TRY(cudaEventRecord(ev_join, aux));
    KM_CUDA_TRY(cudaStreamWaitEvent(stream, ev_join, 0));
  } else {
    if (copy || !on_device)
      KM_CUDA_TRY(cudaMemcpyAsync(X_owned, Xsrc, bytes,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
    const int blocks = (int)std::min<uint64_t>((n + 7) / 8, (uint64_t)num_sms * 16);
    prep_points_kernel<<<blocks, 256, 0, stream>>>(X, n, d, dp, xn2, xn2d, Xb, Xlo, st);
  }
  KM_CUDA_TRY(cudaGetLastError());
  reduce_f64_partial_kernel<<<256, 256, 0, stream>>>(xn2d, n, red_part);
  reduce_f64_final_kernel<<<1, 32, 0, stream>>>(red_part, 256, &st->sum_x2);
  KM_CUDA_TRY(cudaGetLastError());
  if (precision != KM_PREC_FP32) {
    KM_TRY(encode_tmap_bf16(&tmA, Xb, dp, n, 64, 128));
    const uint32_t bbox = tc.chunked ? tc.NC : kp;    // rows of one B load
    KM_TRY(encode_tmap_bf16(&tmB, Cb, dp, kp, 64, bbox));
    if (precision == KM_PREC_BF16X3) {
      KM_TRY(encode_tmap_bf16(&tmAlo, Xlo, dp, n, 64, 128));
      KM_TRY(encode_tmap_bf16(&tmBlo, Clo, dp, kp, 64, bbox));
    } else {
      tmAlo = tmA;
      tmBlo = tmB;
    }
  }
  KM_TRY(read_state());
  if (h_st->err & KM_DEVERR_NONFINITE) return KM_ERR_ARG;
  a_exact = h_st->x_not_bf16 == 0u;
  tb = make_tie_bound(precision, d, a_exact);
  if (precision == KM_PREC_BF16X3) tc_mode = a_exact ? TC_SPLIT2 : TC_SPLIT3;
  data_ready = true;
  return KM_OK;
}

namespace {
__global__ void bf16_decode_kernel(const uint16_t* __restrict__ src, uint64_t count, float* __restrict__ dst) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = __uint_as_float((uint32_t)src[i] << 16);
}
}  // namespace

km_status LloydEngine::set_points_bf16(const uint16_t* Xsrc, bool on_device) {
  KM_CUDA_TRY(cudaSetDevice(device));
  if (!X_owned) KM_TRY(dalloc(&X_owned, (size_t)n * d));
  const uint64_t count = n * (uint64_t)d;
  const uint16_t* src = Xsrc;
  uint16_t* tmp = nullptr;
  if (!on_device) {
    // host BF16 bits go to a staging buffer (half the bytes of the FP32 copy)
    KM_TRY(dalloc(&tmp, count));
    KM_CUDA_TRY(cudaMemcpyAsync(tmp, Xsrc, sizeof(uint16_t) * count, cudaMemcpyHostToDevice, stream));
    src = tmp;
  }
  const unsigned blocks = (unsigned)std::min<uint64_t>((count + 255) / 256, (uint64_t)num_sms * 32);
  bf16_decode_kernel<<<blocks, 256, 0, stream>>>(src, count, X_owned);
  cudaError_t le = cudaGetLastError();
  if (tmp) {
    cudaError_t se = cudaStreamSynchronize(stream);
    cudaFree(tmp);
    KM_CUDA_TRY(le);
    KM_CUDA_TRY(se);
  }
  KM_CUDA_TRY(le);
  return set_points(X_owned, true, false);
}

km_status LloydEngine::reset_state() {
  // Keep sum_x2 (computed at set_points); zero everything else.
  KM_TRY(read_state());
  const double sx = h_st->sum_x2;
  std::memset(h_st, 0, sizeof(DevState));
  h_st->sum_x2 = sx;
  KM_CUDA_TRY(cudaMemcpyAsync(st, h_st, sizeof(DevState), cudaMemcpyHostToDevice, stream));
  KM_CUDA_TRY(cudaStreamSynchronize(stream));
  return KM_OK;
}

km_status LloydEngine::set_centroids_dev(const float* Csrc) {
  if (Csrc != C)
    KM_CUDA_TRY(cudaMemcpyAsync(C, Csrc, sizeof(float) * k * d, cudaMemcpyDeviceToDevice, stream));
  KM_CUDA_TRY(cudaMemsetAsync(&st->cmax, 0, sizeof(float), stream));
  const uint32_t kp64 = (kp + 63) & ~63u;
  const int blocks = (int)((kp64 * 32 + 255) / 256);
  prep_centroids_kernel<<<blocks, 256, 0, stream>>>(C, k, kp, d, dp, cn2, Cb, Clo, Ct, st, kp64);
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status LloydEngine::enqueue_distance(float* Dout) {
  if (precision == KM_PREC_FP32) {
    KM_TRY(launch_assign_f32(X, C, cn2, xn2, n, d, k, tb, st, labels, mindist, rq, Dout, stream));
  } else {
    KM_TRY(launch_assign_tc(tc, tc_mode, tmA, tmAlo, tmB, tmBlo, cn2, xn2, n, k,
                            kp, tb, st, labels, mindist, rq, Dout, stream));
  }
  return KM_OK;
}

km_status LloydEngine::enqueue_refine() {
  if (rq.wide)
    return launch_refine_gemm(refine_v4, num_sms, X, C, Ct, cn2, xn2, n, d, k, tb32, st, rq, rq2, fidx,
                              nfull, labels, mindist, stream);
  return launch_refine(refine_v4, num_sms, X, C, Ct, d, k, st, rq, labels, mindist, stream);
}

km_status LloydEngine::enqueue_assign(float* Dout) {
  KM_TRY(enqueue_distance(Dout));
  return enqueue_refine();
}

km_status LloydEngine::enqueue_finalize(const LoopConsts& lc) {
  KM_CUDA_TRY(launch_pdl(finalize_kernel, (k * 32 + 255) / 256, 256, 0, stream, Cn, C, dsq, objpart, counts,
                         lc.empty, d, dp, k, lc.tol, cn2, Cb, Clo, Ct, shift_c, obj_c, st, lc));
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status LloydEngine::enqueue_sort(const uint32_t* lab) {
  const unsigned hb = (nseg + sort_wpb - 1) / sort_wpb;
  // programmatic dependent launches: each kernel waits for its predecessor
  // (griddepcontrol.wait) before reading, but is scheduled while it drains
  KM_CUDA_TRY(launch_pdl(seg_hist_kernel, hb, sort_wpb * 32, sort_smem, stream, lab, n, k, seg, nseg, seghist, st));
  // per-cluster segment scans; the last block also scans the cluster counts
  KM_CUDA_TRY(launch_pdl(seg_scan_kernel, (k * 32 + 511) / 512, 512, 0, stream, seghist, k, nseg, counts, st,
                         cstart, k <= 1024u ? order : (uint32_t*)nullptr));
  KM_CUDA_TRY(launch_pdl(seg_scatter_kernel, hb, sort_wpb * 32, sort_smem, stream, lab, n, k, seg, nseg, seghist,
                         cstart, perm, st));
  KM_CUDA_TRY(cudaGetLastError());
  return KM_OK;
}

km_status LloydEngine::enqueue_update_step(float tol) {
  (void)tol;
  return launch_update_sums(X, perm, cstart, d, k, C, Cn, dsq, objpart, st, stream,
                            k <= 1024u ? order : nullptr);
}

km_status LloydEngine::enqueue_iteration(const LoopConsts& lc) {
  KM_TRY(enqueue_assign(nullptr));
  KM_TRY(enqueue_sort(labels));
  KM_TRY(enqueue_update_step(lc.tol));
  return enqueue_finalize(lc);
}

km_status LloydEngine::read_state() {
  KM_CUDA_TRY(cudaMemcpyAsync(h_st, st, sizeof(DevState), cudaMemcpyDeviceToHost, stream));
  KM_CUDA_TRY(cudaStreamSynchronize(stream));
  return KM_OK;
}

km_status LloydEngine::check_device_error() {
  KM_TRY(read_state());
  return status_of_device_error(h_st->err);
}

}  // namespace km
