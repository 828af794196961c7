// Link-compatible replacements of FINUFFT's type-1 entry points, the boundary MP_TOOLS calls
// at code/src/mp_sqom56.f90:1148 (finufft2d1, once per frame and species) and
// code/src/mp_sql56.f90:1129 (once per z-layer).  Host arrays in and out; the call is
// synchronous and retains no caller pointer.  Plans, device buffers and pinned host staging
// buffers are cached across calls (mp_sqom repeats identical (n_qx, n_qy, eps, iflag) calls for
// every frame): the caller's (pageable) arrays are copied into pinned memory on the host, moved
// by one asynchronous copy each way, and the call synchronises once, reading the modes and the
// device error flag together.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "mpsq_internal.h"

using namespace mpsq;

namespace {

struct CachedPlan {
  mpsq_nufft_plan* plan = nullptr;
  int dim = 0, iflag = 0, prec = 0;
  int64_t m[3] = {0, 0, 0};
  double eps = 0;
};

struct DropinState {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  CachedPlan cache[4];
  int next = 0;
  void* dpts = nullptr;  // x, y, z staging
  size_t dpts_bytes = 0;
  void* dfk = nullptr;
  size_t dfk_bytes = 0;
  void* hin = nullptr;   // pinned host staging of the inputs (x, y, z, c)
  size_t hin_bytes = 0;
  void* hout = nullptr;  // pinned host staging of the modes, then the error flag
  size_t hout_bytes = 0;
  bool warned = false;
};

DropinState& state() {
  static DropinState* s = new DropinState();  // never destroyed: safe at process exit
  return *s;
}

int grow(void** p, size_t* have, size_t need) {
  if (need <= *have) return MPSQ_OK;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  MPSQ_CUDA_TRY(cudaMalloc(p, need));
  *have = need;
  return MPSQ_OK;
}

int grow_pinned(void** p, size_t* have, size_t need) {
  if (need <= *have) return MPSQ_OK;
  cudaFreeHost(*p);
  *p = nullptr;
  *have = 0;
  MPSQ_CUDA_TRY(cudaHostAlloc(p, need, cudaHostAllocDefault));
  *have = need;
  return MPSQ_OK;
}

int get_plan(DropinState& st, int dim, const int64_t* m, int iflag, double eps, int prec,
             mpsq_nufft_plan** out) {
  for (auto& c : st.cache) {
    if (c.plan && c.dim == dim && c.iflag == iflag && c.prec == prec && c.eps == eps &&
        c.m[0] == m[0] && c.m[1] == m[1] && (dim == 2 || c.m[2] == m[2])) {
      *out = c.plan;
      return MPSQ_OK;
    }
  }
  CachedPlan& c = st.cache[st.next];
  st.next = (st.next + 1) % 4;
  if (c.plan) mpsq_nufft_destroy(c.plan);
  c.plan = nullptr;
  int rc = mpsq_nufft_makeplan(dim, m, iflag, 1, eps, prec, st.stream, &c.plan);
  if (rc) return rc;
  c.dim = dim;
  c.iflag = iflag;
  c.prec = prec;
  c.eps = eps;
  c.m[0] = m[0];
  c.m[1] = m[1];
  c.m[2] = dim == 3 ? m[2] : 1;
  *out = c.plan;
  return MPSQ_OK;
}



template <typename T>
int run_type1(int dim, int64_t nj, const T* x, const T* y, const T* z, const T* c, int iflag,
              double eps, const int64_t* m, T* fk) {
  if (nj < 0) return fail(MPSQ_ERR_ARG, "finufft type 1: nj < 0");
  for (int k = 0; k < dim; ++k)
    if (m[k] < 0) return fail(MPSQ_ERR_ARG, "finufft type 1: negative mode count");
  int64_t nm = 1;
  for (int k = 0; k < dim; ++k) nm *= m[k];
  if (nm == 0) return MPSQ_OK;  // nothing to compute
  if (!fk) return fail(MPSQ_ERR_ARG, "finufft type 1: null fk");
  if (nj > 0 && (!x || !y || (dim == 3 && !z) || !c))
    return fail(MPSQ_ERR_ARG, "finufft type 1: null input array");
  const int prec = sizeof(T) == 8 ? MPSQ_FP64 : MPSQ_FP32;
  DropinState& st = state();
  std::lock_guard<std::mutex> lock(st.mu);
  if (!st.stream) MPSQ_CUDA_TRY(cudaStreamCreateWithFlags(&st.stream, cudaStreamNonBlocking));
  mpsq_nufft_plan* plan = nullptr;
  int rc = get_plan(st, dim, m, iflag, eps, prec, &plan);
  if (rc) return rc;
  // inputs in one block [x | y | z | c] (z only in 3D), device and pinned host alike; every
  // segment starts on a 256-byte boundary (the strengths are read as 8- or 16-byte complex)
  const size_t n1 = (size_t)std::max<int64_t>(nj, 1);
  const size_t seg = (sizeof(T) * n1 + 255) & ~size_t(255);       // one coordinate array
  const size_t off_c = (size_t)dim * seg;
  const size_t in_bytes = off_c + 2 * sizeof(T) * n1;
  const size_t fk_bytes = 2 * sizeof(T) * (size_t)nm;
  const size_t flag_off = (fk_bytes + 15) & ~size_t(15);
  rc = grow(&st.dpts, &st.dpts_bytes, in_bytes);
  if (!rc) rc = grow(&st.dfk, &st.dfk_bytes, fk_bytes);
  if (!rc) rc = grow_pinned(&st.hin, &st.hin_bytes, in_bytes);
  if (!rc) rc = grow_pinned(&st.hout, &st.hout_bytes, flag_off + sizeof(int));
  if (rc) return rc;
  char* const dbase = (char*)st.dpts;
  T* dx = (T*)dbase;
  T* dy = (T*)(dbase + seg);
  T* dz = (T*)(dbase + 2 * seg);
  T* dc = (T*)(dbase + off_c);
  cudaStream_t s = st.stream;
  if (nj > 0) {
    char* const hbase = (char*)st.hin;
    memcpy(hbase, x, sizeof(T) * nj);
    memcpy(hbase + seg, y, sizeof(T) * nj);
    if (dim == 3) memcpy(hbase + 2 * seg, z, sizeof(T) * nj);
    memcpy(hbase + off_c, c, 2 * sizeof(T) * nj);
    MPSQ_CUDA_TRY(cudaMemcpyAsync(dbase, hbase, in_bytes, cudaMemcpyHostToDevice, s));
  }
  rc = mpsq_nufft_setpts(plan, nj, dx, dy, dim == 3 ? dz : nullptr);
  if (!rc) rc = mpsq_nufft_execute(plan, dc, st.dfk);
  if (rc) return rc;
  char* hout = (char*)st.hout;
  MPSQ_CUDA_TRY(cudaMemcpyAsync(hout, st.dfk, fk_bytes, cudaMemcpyDeviceToHost, s));
  MPSQ_CUDA_TRY(cudaMemcpyAsync(hout + flag_off, plan_error_flag(plan), sizeof(int),
                                cudaMemcpyDeviceToHost, s));
  MPSQ_CUDA_TRY(cudaStreamSynchronize(s));
  int flag = 0;
  memcpy(&flag, hout + flag_off, sizeof(int));
  rc = dev_error_status(flag);
  if (rc) return rc;
  memcpy(fk, hout, fk_bytes);
  return MPSQ_OK;
}

int report(int rc) {
  // The reference never inspects ier (mp_sqom56.f90:1148-1154): make failures visible once.
  if (rc) {
    DropinState& st = state();
    if (!st.warned) {
      fprintf(stderr, "mpsq: finufft replacement failed (code %d): %s\n", rc, mpsq_last_error());
      st.warned = true;
    }
  }
  return rc;
}

}  // namespace

extern "C" int finufft2d1(int64_t nj, double* xj, double* yj, double* cj, int iflag, double eps,
                          int64_t ms, int64_t mt, double* fk, void* opts) {
  (void)opts;
  const int64_t m[3] = {ms, mt, 1};
  return report(run_type1<double>(2, nj, xj, yj, nullptr, cj, iflag, eps, m, fk));
}

extern "C" int finufft3d1(int64_t nj, double* xj, double* yj, double* zj, double* cj, int iflag,
                          double eps, int64_t ms, int64_t mt, int64_t mu, double* fk, void* opts) {
  (void)opts;
  const int64_t m[3] = {ms, mt, mu};
  return report(run_type1<double>(3, nj, xj, yj, zj, cj, iflag, eps, m, fk));
}

extern "C" int finufftf2d1(int64_t nj, float* xj, float* yj, float* cj, int iflag, float eps,
                           int64_t ms, int64_t mt, float* fk, void* opts) {
  (void)opts;
  const int64_t m[3] = {ms, mt, 1};
  return report(run_type1<float>(2, nj, xj, yj, nullptr, cj, iflag, eps, m, fk));
}

extern "C" int finufftf3d1(int64_t nj, float* xj, float* yj, float* zj, float* cj, int iflag,
                           float eps, int64_t ms, int64_t mt, int64_t mu, float* fk, void* opts) {
  (void)opts;
  const int64_t m[3] = {ms, mt, mu};
  return report(run_type1<float>(3, nj, xj, yj, zj, cj, iflag, eps, m, fk));
}

extern "C" void finufft2d1_(const int64_t* nj, const double* xj, const double* yj,
                            const double* cj, const int* iflag, const double* eps,
                            const int64_t* ms, const int64_t* mt, double* fk, const void* opts,
                            int* ier) {
  (void)opts;
  int rc;
  if (!nj || !iflag || !eps || !ms || !mt)
    rc = report(fail(MPSQ_ERR_ARG, "finufft2d1_: null scalar argument"));
  else {
    const int64_t m[3] = {*ms, *mt, 1};
    rc = report(run_type1<double>(2, *nj, xj, yj, nullptr, cj, *iflag, *eps, m, fk));
  }
  if (ier) *ier = rc;
}

extern "C" void finufft3d1_(const int64_t* nj, const double* xj, const double* yj,
                            const double* zj, const double* cj, const int* iflag,
                            const double* eps, const int64_t* ms, const int64_t* mt,
                            const int64_t* mu, double* fk, const void* opts, int* ier) {
  (void)opts;
  int rc;
  if (!nj || !iflag || !eps || !ms || !mt || !mu)
    rc = report(fail(MPSQ_ERR_ARG, "finufft3d1_: null scalar argument"));
  else {
    const int64_t m[3] = {*ms, *mt, *mu};
    rc = report(run_type1<double>(3, *nj, xj, yj, zj, cj, *iflag, *eps, m, fk));
  }
  if (ier) *ier = rc;
}
