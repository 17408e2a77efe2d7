// capi.cu -- thin C-ABI layer (the role cuda_api.cu plays in the reference):
// argument validation, host<->device staging on the library stream, status
// codes and error strings.  All arithmetic happens in the kernels of
// fp64_kernels.cu, split_kernels.cu and front_end.cu; there is no host
// compute path.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "common.cuh"

namespace rimp2 {

static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches{0};
static cudaStream_t g_user_stream = nullptr;
static cudaStream_t g_lib_stream = nullptr;
static std::mutex g_mu;
static int g_dev_ok = -1;  // -1 unknown, 0 no, 1 yes
static int *g_dev_err = nullptr;
static bool g_timing = false;
static float g_times[4] = {0, 0, 0, 0};

int *device_error_word() { return g_dev_err; }
bool timing_enabled() { return g_timing; }
void record_timing(int slot, float ms) {
  if (slot >= 0 && slot < 4) g_times[slot] = ms;
}

int collect_device_error(cudaStream_t s) {
  RIMP2_CK(cudaStreamSynchronize(s));
  int h = 0;
  RIMP2_CK(cudaMemcpy(&h, g_dev_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    RIMP2_CK(cudaMemset(g_dev_err, 0, sizeof(int)));
    set_error("a device-side bounded wait expired (code %d); the kernel returned early", h);
    return RIMP2_ERR_TIMEOUT;
  }
  return RIMP2_OK;
}

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }
void count_launch(int n) { g_launches += n; }
static std::atomic<int> g_last_split_kernel{0};
void note_split_kernel(int k) { g_last_split_kernel = k; }

bool inject_fault(const char *what) {
  const char *v = getenv("RIMP2_FAULT_INJECT");
  return v && strcmp(v, what) == 0;
}

int DevBuf::alloc(size_t bytes, cudaStream_t st) {
  s = st;
  n = bytes;
  if (bytes == 0) bytes = 16;
  if (inject_fault("alloc")) {
    set_error("injected device allocation failure (RIMP2_FAULT_INJECT=alloc)");
    return RIMP2_ERR_NOMEM;
  }
  cudaError_t e = cudaMallocAsync(&p, bytes, st);
  if (e != cudaSuccess) {
    p = nullptr;
    set_error("device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    return RIMP2_ERR_NOMEM;
  }
  return RIMP2_OK;
}

int ensure_device() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_dev_ok == 1) return RIMP2_OK;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    (void)cudaGetLastError();
    set_error("no CUDA device available (%s); this library has no CPU path",
              e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    g_dev_ok = 0;
    return RIMP2_ERR_NODEV;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    set_error("cudaGetDeviceProperties failed");
    return RIMP2_ERR_NODEV;
  }
  if (!(prop.major == 10 && prop.minor == 3)) {
    set_error("device %s is sm_%d%d; this library is built for sm_103a (GB300) only", prop.name,
              prop.major, prop.minor);
    g_dev_ok = 0;
    return RIMP2_ERR_NODEV;
  }
  if (!g_lib_stream) {
    if (cudaStreamCreateWithFlags(&g_lib_stream, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("stream creation failed");
      return RIMP2_ERR_CUDA;
    }
  }
  if (!g_dev_err) {
    if (cudaMalloc(&g_dev_err, sizeof(int)) != cudaSuccess ||
        cudaMemset(g_dev_err, 0, sizeof(int)) != cudaSuccess) {
      set_error("error-word allocation failed");
      return RIMP2_ERR_NOMEM;
    }
  }
  // keep freed stream-ordered scratch in the pool between calls instead of
  // returning it to the driver at every synchronisation
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  // load the allocation-free entry point's fixed array and kernels now, while
  // the caller can still spare the memory; a failure here only concerns that
  // entry point, which reports its own error when called
  if (noalloc_preload() != RIMP2_OK) clear_error();
  g_dev_ok = 1;
  return RIMP2_OK;
}

cudaStream_t current_stream() { return g_user_stream ? g_user_stream : g_lib_stream; }

static cudaStream_t g_copy_stream = nullptr;
cudaStream_t copy_stream() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_copy_stream) cudaStreamCreateWithFlags(&g_copy_stream, cudaStreamNonBlocking);
  return g_copy_stream;
}

static cudaStream_t g_slice_stream = nullptr;
cudaStream_t slice_stream() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_slice_stream) cudaStreamCreateWithFlags(&g_slice_stream, cudaStreamNonBlocking);
  return g_slice_stream;
}

}  // namespace rimp2

using namespace rimp2;

namespace {

int h2d(DevBuf &b, const double *h, size_t n, cudaStream_t s) {
  RIMP2_TRY(b.alloc(n * sizeof(double), s));
  RIMP2_CK(cudaMemcpyAsync(b.p, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
  return RIMP2_OK;
}
int dalloc(DevBuf &b, size_t n, cudaStream_t s) { return b.alloc(n * sizeof(double), s); }
int d2h(double *h, const DevBuf &b, size_t n, cudaStream_t s) {
  RIMP2_CK(cudaMemcpyAsync(h, b.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  return RIMP2_OK;
}
int finish(cudaStream_t s) {
  RIMP2_CK(cudaStreamSynchronize(s));
  RIMP2_CK(cudaGetLastError());
  return collect_device_error(s);
}

GemmDesc gd() {
  GemmDesc g;
  memset(&g, 0, sizeof g);
  g.alpha = 1.0;
  g.beta = 0.0;
  g.nb0 = g.nb1 = 1;
  return g;
}

// --- device-pointer building blocks ------------------------------------------

// X(i,j,a,b) = g_ij(a,b) / D  (RIMP2.F90:397-404), X layout (nocc,nocc,nvirt,nvirt)
int dev_g_over_d(int nvirt, int nocc, int NBA, const double *Ca, const double *eo,
                 const double *ev, double *X, cudaStream_t s) {
  GemmDesc g = gd();
  const long long no = nocc, nv = nvirt, nb = NBA;
  g.M = nvirt;
  g.N = nvirt;
  g.K = NBA;
  g.A = Ca;
  g.sAm = nb;
  g.sAk = 1;
  g.sAb0 = nb * nv;
  g.B = Ca;
  g.sBk = 1;
  g.sBn = nb;
  g.sBb1 = nb * nv;
  g.C = X;
  g.sCm = no * no;
  g.sCn = no * no * nv;
  g.sCb0 = 1;
  g.sCb1 = no;
  g.nb0 = nocc;
  g.nb1 = nocc;
  g.eo = eo;
  g.ev = ev;
  g.denom = 1;
  return launch_gemm_f64(g, s);
}

int dev_tocca(int nvirt, int nocc, int noccEOS, int NBA, const double *Ca, const double *eo,
              const double *ev, double *tocc, const double *U, cudaStream_t s) {
  DevBuf X;
  const size_t no = nocc, nv = nvirt;
  RIMP2_TRY(dalloc(X, no * no * nv * nv, s));
  RIMP2_TRY(dev_g_over_d(nvirt, nocc, NBA, Ca, eo, ev, X.as<double>(), s));
  // tocc(i,jL,ab) = sum_j X(i,j,ab) U(j,jL)   (RIMP2.F90:406-412)
  GemmDesc g = gd();
  g.M = nvirt * nvirt;
  g.N = noccEOS;
  g.K = nocc;
  g.A = X.as<double>();
  g.sAm = (long long)no * no;
  g.sAk = nocc;
  g.sAb0 = 1;
  g.B = U;
  g.sBk = 1;
  g.sBn = nocc;
  g.C = tocc;
  g.sCm = (long long)no * noccEOS;
  g.sCn = nocc;
  g.sCb0 = 1;
  g.nb0 = nocc;
  return launch_gemm_f64(g, s);
}

int dev_tvirta(int nvirt, int nocc, int nvirtEOS, int NBA, const double *Ca, const double *eo,
               const double *ev, double *tvirt, const double *U, cudaStream_t s) {
  DevBuf X;
  const long long no = nocc, nv = nvirt;
  RIMP2_TRY(dalloc(X, (size_t)(no * no * nv * nv), s));
  RIMP2_TRY(dev_g_over_d(nvirt, nocc, NBA, Ca, eo, ev, X.as<double>(), s));
  // tvirt(i,j,aL,b) = sum_a X(i,j,a,b) U(a,aL)   (RIMP2.F90:442-448)
  GemmDesc g = gd();
  g.M = nocc * nocc;
  g.N = nvirtEOS;
  g.K = nvirt;
  g.A = X.as<double>();
  g.sAm = 1;
  g.sAk = no * no;
  g.sAb0 = no * no * nv;
  g.B = U;
  g.sBk = 1;
  g.sBn = nv;
  g.C = tvirt;
  g.sCm = 1;
  g.sCn = no * no;
  g.sCb0 = no * no * nvirtEOS;
  g.nb0 = nvirt;
  return launch_gemm_f64(g, s);
}

int dev_toccb(int nvirt, int noccEOS, const double *tocc, const double *UvirtT, double *toccEOS,
              cudaStream_t s) {
  GemmDesc g = gd();
  const long long nv = nvirt, ne = noccEOS;
  g.M = nvirt;
  g.N = noccEOS;
  g.K = nvirt;
  g.A = UvirtT;
  g.sAm = nv;
  g.sAk = 1;
  g.B = tocc;
  g.sBk = ne * ne;
  g.sBn = 1;
  g.sBb0 = ne;
  g.sBb1 = ne * ne * nv;
  g.C = toccEOS;
  g.sCm = 1;
  g.sCn = nv;
  g.sCb0 = nv * ne * nv;
  g.sCb1 = nv * ne;
  g.nb0 = noccEOS;
  g.nb1 = nvirt;
  return launch_gemm_f64(g, s);
}

int dev_tvirtb(int nvirtEOS, int nocc, const double *tvirt, const double *UoccT, double *tvirtEOS,
               cudaStream_t s) {
  GemmDesc g = gd();
  const long long ve = nvirtEOS, no = nocc;
  g.M = nocc;
  g.N = nocc;
  g.K = nocc;
  g.A = tvirt;
  g.sAm = 1;
  g.sAk = no;
  g.sAb0 = no * no;
  g.sAb1 = no * no * ve;
  g.B = UoccT;
  g.sBk = 1;
  g.sBn = no;
  g.C = tvirtEOS;
  g.sCm = ve;
  g.sCn = ve * no * ve;
  g.sCb0 = 1;
  g.sCb1 = ve * no;
  g.nb0 = nvirtEOS;
  g.nb1 = nvirtEOS;
  return launch_gemm_f64(g, s);
}

int dev_transalpha2(int n2, int n1, int n3, int nba, const double *U, const double *CD4,
                    double *CD5, cudaStream_t s) {
  GemmDesc g = gd();
  const long long b = nba;
  g.M = nba;
  g.N = n3;
  g.K = n1;
  g.A = CD4;
  g.sAm = 1;
  g.sAk = b;
  g.sAb0 = b * n1;
  g.B = U;
  g.sBk = 1;
  g.sBn = n1;
  g.C = CD5;
  g.sCm = 1;
  g.sCn = b;
  g.sCb0 = b * n3;
  g.nb0 = n2;
  return launch_gemm_f64(g, s);
}

int dev_gen4dimfo(int NBA, const double *X, int n1, int n2, const double *Y, int n3, int n4,
                  double *out, cudaStream_t s) {
  GemmDesc g = gd();
  const long long m = (long long)n1 * n2, n = (long long)n3 * n4;
  if (m > 2147483647LL || n > 2147483647LL) {
    set_error("gen4dimfo extents too large");
    return RIMP2_ERR_ARG;
  }
  g.M = (int)m;
  g.N = (int)n;
  g.K = NBA;
  g.A = X;
  g.sAm = NBA;
  g.sAk = 1;
  g.B = Y;
  g.sBk = 1;
  g.sBn = NBA;
  g.C = out;
  g.sCm = 1;
  g.sCn = m;
  return launch_gemm_f64(g, s);
}

int dev_dgemm(char ta, char tb, int M, int N, int K, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *Cm, int ldc, cudaStream_t s) {
  GemmDesc g = gd();
  const bool tA = (ta == 'T' || ta == 't' || ta == 'C' || ta == 'c');
  const bool tB = (tb == 'T' || tb == 't' || tb == 'C' || tb == 'c');
  g.M = M;
  g.N = N;
  g.K = K;
  g.alpha = alpha;
  g.beta = beta;
  g.A = A;
  g.sAm = tA ? lda : 1;
  g.sAk = tA ? 1 : lda;
  g.B = B;
  g.sBk = tB ? ldb : 1;
  g.sBn = tB ? 1 : ldb;
  g.C = Cm;
  g.sCm = 1;
  g.sCn = ldc;
  return launch_gemm_f64(g, s);
}

bool pos(const int *p) { return p && *p > 0; }

// TransAlpha2 with the transformation matrix given by strides:
// CD5(al,n3,n2) = sum_n1 U(n1,n3) CD4(al,n1,n2), U(k,n) = U[k*sUk + n*sUn]
int dev_transalpha2_strided(int n2, int n1, int n3, int nba, const double *U, long long sUk,
                            long long sUn, const double *CD4, double *CD5, cudaStream_t s) {
  GemmDesc g = gd();
  const long long b = nba;
  g.M = nba;
  g.N = n3;
  g.K = n1;
  g.A = CD4;
  g.sAm = 1;
  g.sAk = b;
  g.sAb0 = b * n1;
  g.B = U;
  g.sBk = sUk;
  g.sBn = sUn;
  g.C = CD5;
  g.sCm = 1;
  g.sCn = b;
  g.sCb0 = b * n3;
  g.nb0 = n2;
  return launch_gemm_f64(g, s);
}

// max |P(i,j) - delta_ij| over an n x n matrix (one block)
__global__ void identity_dev_kernel(const double *P, int n, double *out) {
  __shared__ double red[32];
  double m = 0.0;
  const long long nn = (long long)n * n;
  for (long long t = threadIdx.x; t < nn; t += blockDim.x) {
    const long long i = t % n, j = t / n;
    m = fmax(m, fabs(P[t] - (i == j ? 1.0 : 0.0)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    *out = r;
  }
}

// true if P = I within 1e-13 (P on the device; synchronises s)
int is_identity(const double *P, int n, double *dwork, bool *yes, cudaStream_t s) {
  identity_dev_kernel<<<1, 1024, 0, s>>>(P, n, dwork);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  double h = 1.0;
  RIMP2_CK(cudaMemcpyAsync(&h, dwork, sizeof h, cudaMemcpyDeviceToHost, s));
  RIMP2_CK(cudaStreamSynchronize(s));
  *yes = (h <= 1e-13);
  return RIMP2_OK;
}

}  // namespace

extern "C" {

const char *rimp2_last_error_string(void) { return g_err; }
const char *rimp2_version(void) { return "rimp2_gpu_gb300 0.1 (sm_103a)"; }
long long rimp2_kernel_launch_count(void) { return g_launches.load(); }

int rimp2_sync_status(void *stream) {
  clear_error();
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  RIMP2_CK(cudaGetLastError());
  return collect_device_error(s);
}

int rimp2_selftest_bounded_wait(long long budget_cycles, void *stream) {
  clear_error();
  RIMP2_REQ(budget_cycles > 0 && budget_cycles <= 1000000000LL,
            "rimp2_selftest_bounded_wait: budget must be in (0, 1e9] cycles");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return bounded_wait_selftest(budget_cycles, s);
}

int rimp2_selftest_rcp_denom(int n, const float *d, float *r, float *ref) {
  clear_error();
  RIMP2_REQ(n > 0 && n <= (1 << 26) && d && r && ref,
            "rimp2_selftest_rcp_denom: need 0 < n <= 2^26 and three host arrays");
  RIMP2_TRY(ensure_device());
  return rcp_denom_selftest(n, d, r, ref, current_stream());
}

int rimp2_set_timing(int on) {
  g_timing = (on != 0);
  return RIMP2_OK;
}

int rimp2_last_split_kernel(void) { return g_last_split_kernel.load(); }

int rimp2_last_timing(float *ms4) {
  if (!ms4) return RIMP2_ERR_ARG;
  for (int k = 0; k < 4; ++k) ms4[k] = g_times[k];
  return RIMP2_OK;
}

int rimp2_probe_fp64_peak(double *tflops) {
  clear_error();
  RIMP2_REQ(tflops, "rimp2_probe_fp64_peak: null argument");
  RIMP2_TRY(ensure_device());
  return probe_fp64_peak(tflops, current_stream());
}

int rimp2_set_stream(void *stream) {
  g_user_stream = (cudaStream_t)stream;
  return RIMP2_OK;
}

int rimp2_get_dev_mem(size_t *total, size_t *free_bytes) {
  clear_error();
  RIMP2_REQ(total && free_bytes, "rimp2_get_dev_mem: null argument");
  RIMP2_TRY(ensure_device());
  RIMP2_CK(cudaMemGetInfo(free_bytes, total));
  return RIMP2_OK;
}

int rimp2_calc_tocca(const int *nvirt, const int *nocc, const int *noccEOS, const int *NBA,
                     const double *Calpha, const double *EVocc, const double *EVvirt, double *tocc,
                     const double *UoccEOST) {
  clear_error();
  RIMP2_REQ(pos(nvirt) && pos(nocc) && pos(noccEOS) && pos(NBA), "rimp2_calc_tocca: bad dims");
  RIMP2_REQ(Calpha && EVocc && EVvirt && tocc && UoccEOST, "rimp2_calc_tocca: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nv = *nvirt, no = *nocc, ne = *noccEOS, nb = *NBA;
  DevBuf dC, deo, dev, dU, dT;
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(deo, EVocc, no, s));
  RIMP2_TRY(h2d(dev, EVvirt, nv, s));
  RIMP2_TRY(h2d(dU, UoccEOST, no * ne, s));
  RIMP2_TRY(dalloc(dT, no * ne * nv * nv, s));
  RIMP2_TRY(dev_tocca(*nvirt, *nocc, *noccEOS, *NBA, dC.as<double>(), deo.as<double>(),
                      dev.as<double>(), dT.as<double>(), dU.as<double>(), s));
  RIMP2_TRY(d2h(tocc, dT, no * ne * nv * nv, s));
  return finish(s);
}

int rimp2_calc_tvirta(const int *nvirt, const int *nocc, const int *nvirtEOS, const int *NBA,
                      const double *Calpha, const double *EVocc, const double *EVvirt,
                      double *tvirt, const double *UvirtEOST) {
  clear_error();
  RIMP2_REQ(pos(nvirt) && pos(nocc) && pos(nvirtEOS) && pos(NBA), "rimp2_calc_tvirta: bad dims");
  RIMP2_REQ(Calpha && EVocc && EVvirt && tvirt && UvirtEOST, "rimp2_calc_tvirta: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nv = *nvirt, no = *nocc, ve = *nvirtEOS, nb = *NBA;
  DevBuf dC, deo, dev, dU, dT;
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(deo, EVocc, no, s));
  RIMP2_TRY(h2d(dev, EVvirt, nv, s));
  RIMP2_TRY(h2d(dU, UvirtEOST, nv * ve, s));
  RIMP2_TRY(dalloc(dT, no * no * ve * nv, s));
  RIMP2_TRY(dev_tvirta(*nvirt, *nocc, *nvirtEOS, *NBA, dC.as<double>(), deo.as<double>(),
                       dev.as<double>(), dT.as<double>(), dU.as<double>(), s));
  RIMP2_TRY(d2h(tvirt, dT, no * no * ve * nv, s));
  return finish(s);
}

int rimp2_calc_toccb(const int *nvirt, const int *noccEOS, const double *tocc,
                     const double *UvirtT, double *toccEOS) {
  clear_error();
  RIMP2_REQ(pos(nvirt) && pos(noccEOS), "rimp2_calc_toccb: bad dims");
  RIMP2_REQ(tocc && UvirtT && toccEOS, "rimp2_calc_toccb: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nv = *nvirt, ne = *noccEOS;
  DevBuf dT, dU, dO;
  RIMP2_TRY(h2d(dT, tocc, ne * ne * nv * nv, s));
  RIMP2_TRY(h2d(dU, UvirtT, nv * nv, s));
  RIMP2_TRY(dalloc(dO, nv * ne * nv * ne, s));
  RIMP2_TRY(dev_toccb(*nvirt, *noccEOS, dT.as<double>(), dU.as<double>(), dO.as<double>(), s));
  RIMP2_TRY(d2h(toccEOS, dO, nv * ne * nv * ne, s));
  return finish(s);
}

int rimp2_calc_tvirtb(const int *nvirtEOS, const int *nocc, const double *tvirt,
                      const double *UoccT, double *tvirtEOS) {
  clear_error();
  RIMP2_REQ(pos(nvirtEOS) && pos(nocc), "rimp2_calc_tvirtb: bad dims");
  RIMP2_REQ(tvirt && UoccT && tvirtEOS, "rimp2_calc_tvirtb: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t ve = *nvirtEOS, no = *nocc;
  DevBuf dT, dU, dO;
  RIMP2_TRY(h2d(dT, tvirt, no * no * ve * ve, s));
  RIMP2_TRY(h2d(dU, UoccT, no * no, s));
  RIMP2_TRY(dalloc(dO, ve * no * ve * no, s));
  RIMP2_TRY(dev_tvirtb(*nvirtEOS, *nocc, dT.as<double>(), dU.as<double>(), dO.as<double>(), s));
  RIMP2_TRY(d2h(tvirtEOS, dO, ve * no * ve * no, s));
  return finish(s);
}

int rimp2_transalpha2(const int *n2, const int *n1, const int *n3, const int *nba, const double *U,
                      const double *AlphaCD4, double *AlphaCD5) {
  clear_error();
  RIMP2_REQ(pos(n2) && pos(n1) && pos(n3) && pos(nba), "rimp2_transalpha2: bad dims");
  RIMP2_REQ(U && AlphaCD4 && AlphaCD5, "rimp2_transalpha2: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t a = *n2, b = *n1, c = *n3, nb = *nba;
  DevBuf dU, d4, d5;
  RIMP2_TRY(h2d(dU, U, b * c, s));
  RIMP2_TRY(h2d(d4, AlphaCD4, nb * b * a, s));
  RIMP2_TRY(dalloc(d5, nb * c * a, s));
  RIMP2_TRY(dev_transalpha2(*n2, *n1, *n3, *nba, dU.as<double>(), d4.as<double>(), d5.as<double>(),
                            s));
  RIMP2_TRY(d2h(AlphaCD5, d5, nb * c * a, s));
  return finish(s);
}

int rimp2_transalpha1(const int *nvirt, const int *noccEOS, const int *nba, const double *UvirtT,
                      const double *AlphaCD4, double *AlphaCD5) {
  // RIMP2_TransAlpha1 is RIMP2_TransAlpha2 with n2=noccEOS, n1=n3=nvirt
  return rimp2_transalpha2(noccEOS, nvirt, nvirt, nba, UvirtT, AlphaCD4, AlphaCD5);
}

int rimp2_calc_gen4dimfo(const int *NBA, const double *Calpha3, const int *n1, const int *n2,
                         const double *Calpha4, const int *n3, const int *n4, double *djik) {
  clear_error();
  RIMP2_REQ(pos(NBA) && pos(n1) && pos(n2) && pos(n3) && pos(n4), "rimp2_calc_gen4dimfo: bad dims");
  RIMP2_REQ(Calpha3 && Calpha4 && djik, "rimp2_calc_gen4dimfo: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nb = *NBA, a = *n1, b = *n2, c = *n3, d = *n4;
  DevBuf dX, dY, dO;
  RIMP2_TRY(h2d(dX, Calpha3, nb * a * b, s));
  const double *yp = dX.as<double>();
  if (Calpha4 != Calpha3) {
    RIMP2_TRY(h2d(dY, Calpha4, nb * c * d, s));
    yp = dY.as<double>();
  }
  RIMP2_TRY(dalloc(dO, a * b * c * d, s));
  RIMP2_TRY(dev_gen4dimfo(*NBA, dX.as<double>(), *n1, *n2, yp, *n3, *n4, dO.as<double>(), s));
  RIMP2_TRY(d2h(djik, dO, a * b * c * d, s));
  return finish(s);
}

int rimp2_calc_gocc(const int *nvirt, const int *noccEOS, const int *NBA, const double *Calpha3,
                    double *goccEOS) {
  return rimp2_calc_gen4dimfo(NBA, Calpha3, nvirt, noccEOS, Calpha3, nvirt, noccEOS, goccEOS);
}

int rimp2_calc_gvirt(const int *nvirtEOS, const int *nocc, const int *NBA, const double *Calpha3,
                     double *gvirtEOS) {
  return rimp2_calc_gen4dimfo(NBA, Calpha3, nvirtEOS, nocc, Calpha3, nvirtEOS, nocc, gvirtEOS);
}

int rimp2_dgemm(const char *transa, const char *transb, const int *m, const int *n, const int *k,
                const double *alpha, const double *A, const int *lda, const double *B,
                const int *ldb, const double *beta, double *Cm, const int *ldc) {
  clear_error();
  RIMP2_REQ(transa && transb && m && n && k && alpha && beta && lda && ldb && ldc,
            "rimp2_dgemm: null argument");
  RIMP2_REQ(*m >= 0 && *n >= 0 && *k >= 0, "rimp2_dgemm: negative dims");
  const char ta = *transa, tb = *transb;
  RIMP2_REQ(strchr("NnTtCc", ta) && strchr("NnTtCc", tb), "rimp2_dgemm: bad trans flag");
  const bool tA = !(ta == 'N' || ta == 'n'), tB = !(tb == 'N' || tb == 'n');
  RIMP2_REQ(*lda >= (tA ? (*k > 1 ? *k : 1) : (*m > 1 ? *m : 1)), "rimp2_dgemm: lda too small");
  RIMP2_REQ(*ldb >= (tB ? (*n > 1 ? *n : 1) : (*k > 1 ? *k : 1)), "rimp2_dgemm: ldb too small");
  RIMP2_REQ(*ldc >= (*m > 1 ? *m : 1), "rimp2_dgemm: ldc too small");
  if (*m == 0 || *n == 0) return RIMP2_OK;
  RIMP2_REQ(Cm && (*k == 0 || (A && B)), "rimp2_dgemm: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t na = (size_t)*lda * (tA ? *m : *k), nbb = (size_t)*ldb * (tB ? *k : *n);
  const size_t nc = (size_t)*ldc * *n;
  DevBuf dA, dB, dCc;
  if (*k > 0) {
    RIMP2_TRY(h2d(dA, A, na, s));
    RIMP2_TRY(h2d(dB, B, nbb, s));
  }
  if (*beta != 0.0)
    RIMP2_TRY(h2d(dCc, Cm, nc, s));
  else {
    RIMP2_TRY(dalloc(dCc, nc, s));
    RIMP2_CK(cudaMemsetAsync(dCc.p, 0, nc * sizeof(double), s));
  }
  if (*k > 0) {
    RIMP2_TRY(dev_dgemm(ta, tb, *m, *n, *k, *alpha, dA.as<double>(), *lda, dB.as<double>(), *ldb,
                        *beta, dCc.as<double>(), *ldc, s));
  } else {
    // C = beta*C: a K=0 product, done by the same kernel with a zero sum
    RIMP2_TRY(dev_dgemm(ta, tb, *m, *n, 0, *alpha, dCc.as<double>(), 1, dCc.as<double>(), 1, *beta,
                        dCc.as<double>(), *ldc, s));
  }
  RIMP2_TRY(d2h(Cm, dCc, nc, s));
  return finish(s);
}

int rimp2_steps5to8(const int *nvirt_, const int *nocc_, const int *noccEOS_, const int *nvirtEOS_,
                    const int *NBA_, const double *Calpha, const double *EVocc,
                    const double *EVvirt, const double *UoccEOST, const double *UvirtT,
                    const double *UoccT, const double *UvirtEOST, double *toccEOS,
                    double *tvirtEOS, double *goccEOS, double *gvirtEOS) {
  clear_error();
  RIMP2_REQ(pos(nvirt_) && pos(nocc_) && pos(noccEOS_) && pos(nvirtEOS_) && pos(NBA_),
            "rimp2_steps5to8: bad dims");
  RIMP2_REQ(Calpha && EVocc && EVvirt && UoccEOST && UvirtT && UoccT && UvirtEOST && toccEOS &&
                tvirtEOS && goccEOS && gvirtEOS,
            "rimp2_steps5to8: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const int nvirt = *nvirt_, nocc = *nocc_, noccEOS = *noccEOS_, nvirtEOS = *nvirtEOS_,
            NBA = *NBA_;
  const size_t nv = nvirt, no = nocc, ne = noccEOS, ve = nvirtEOS, nb = NBA;
  DevBuf dC, deo, dev, dUoE, dUvT, dUoT, dUvE;
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(deo, EVocc, no, s));
  RIMP2_TRY(h2d(dev, EVvirt, nv, s));
  RIMP2_TRY(h2d(dUoE, UoccEOST, no * ne, s));
  RIMP2_TRY(h2d(dUvT, UvirtT, nv * nv, s));
  RIMP2_TRY(h2d(dUoT, UoccT, no * no, s));
  RIMP2_TRY(h2d(dUvE, UvirtEOST, nv * ve, s));
  const double *Ca = dC.as<double>(), *eo = deo.as<double>(), *ev = dev.as<double>();
  {  // Step 5 (RIMP2.F90:71-93)
    DevBuf t1, t2, t3, out;
    RIMP2_TRY(dalloc(t1, no * ne * nv * nv, s));
    RIMP2_TRY(dev_tocca(nvirt, nocc, noccEOS, NBA, Ca, eo, ev, t1.as<double>(), dUoE.as<double>(), s));
    RIMP2_TRY(dalloc(t2, ne * ne * nv * nv, s));
    RIMP2_TRY(dev_dgemm('T', 'N', noccEOS, noccEOS * nvirt * nvirt, nocc, 1.0, dUoE.as<double>(),
                        nocc, t1.as<double>(), nocc, 0.0, t2.as<double>(), noccEOS, s));
    RIMP2_TRY(dalloc(t3, nv * nv * ne * ne, s));
    RIMP2_TRY(dev_dgemm('N', 'N', noccEOS * noccEOS * nvirt, nvirt, nvirt, 1.0, t2.as<double>(),
                        noccEOS * noccEOS * nvirt, dUvT.as<double>(), nvirt, 0.0, t3.as<double>(),
                        noccEOS * noccEOS * nvirt, s));
    RIMP2_TRY(dalloc(out, nv * ne * nv * ne, s));
    RIMP2_TRY(dev_toccb(nvirt, noccEOS, t3.as<double>(), dUvT.as<double>(), out.as<double>(), s));
    RIMP2_TRY(d2h(toccEOS, out, nv * ne * nv * ne, s));
    RIMP2_CK(cudaStreamSynchronize(s));
  }
  {  // Step 6 (RIMP2.F90:99-124)
    DevBuf t1, t2, t3, out;
    RIMP2_TRY(dalloc(t1, no * no * ve * nv, s));
    RIMP2_TRY(dev_tvirta(nvirt, nocc, nvirtEOS, NBA, Ca, eo, ev, t1.as<double>(), dUvE.as<double>(), s));
    RIMP2_TRY(dalloc(t2, no * no * ve * ve, s));
    RIMP2_TRY(dev_dgemm('N', 'N', nocc * nocc * nvirtEOS, nvirtEOS, nvirt, 1.0, t1.as<double>(),
                        nocc * nocc * nvirtEOS, dUvE.as<double>(), nvirt, 0.0, t2.as<double>(),
                        nocc * nocc * nvirtEOS, s));
    RIMP2_TRY(dalloc(t3, no * no * ve * ve, s));
    RIMP2_TRY(dev_dgemm('T', 'N', nocc, nocc * nvirtEOS * nvirtEOS, nocc, 1.0, dUoT.as<double>(), nocc,
                        t2.as<double>(), nocc, 0.0, t3.as<double>(), nocc, s));
    RIMP2_TRY(dalloc(out, ve * no * ve * no, s));
    RIMP2_TRY(dev_tvirtb(nvirtEOS, nocc, t3.as<double>(), dUoT.as<double>(), out.as<double>(), s));
    RIMP2_TRY(d2h(tvirtEOS, out, ve * no * ve * no, s));
    RIMP2_CK(cudaStreamSynchronize(s));
  }
  {  // Step 7 (RIMP2.F90:133-147)
    DevBuf c2, c3, out;
    RIMP2_TRY(dalloc(c2, nb * nv * ne, s));
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nvirt, noccEOS, nocc, 1.0, Ca, NBA * nvirt,
                        dUoE.as<double>(), nocc, 0.0, c2.as<double>(), NBA * nvirt, s));
    RIMP2_TRY(dalloc(c3, nb * nv * ne, s));
    RIMP2_TRY(dev_transalpha2(noccEOS, nvirt, nvirt, NBA, dUvT.as<double>(), c2.as<double>(),
                              c3.as<double>(), s));
    RIMP2_TRY(dalloc(out, nv * ne * nv * ne, s));
    RIMP2_TRY(dev_gen4dimfo(NBA, c3.as<double>(), nvirt, noccEOS, c3.as<double>(), nvirt, noccEOS,
                            out.as<double>(), s));
    RIMP2_TRY(d2h(goccEOS, out, nv * ne * nv * ne, s));
    RIMP2_CK(cudaStreamSynchronize(s));
  }
  {  // Step 8 (RIMP2.F90:155-170)
    DevBuf c2, c3, out;
    RIMP2_TRY(dalloc(c2, nb * nv * no, s));
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nvirt, nocc, nocc, 1.0, Ca, NBA * nvirt, dUoT.as<double>(),
                        nocc, 0.0, c2.as<double>(), NBA * nvirt, s));
    RIMP2_TRY(dalloc(c3, nb * ve * no, s));
    RIMP2_TRY(dev_transalpha2(nocc, nvirt, nvirtEOS, NBA, dUvE.as<double>(), c2.as<double>(),
                              c3.as<double>(), s));
    RIMP2_TRY(dalloc(out, ve * no * ve * no, s));
    RIMP2_TRY(dev_gen4dimfo(NBA, c3.as<double>(), nvirtEOS, nocc, c3.as<double>(), nvirtEOS, nocc,
                            out.as<double>(), s));
    RIMP2_TRY(d2h(gvirtEOS, out, ve * no * ve * no, s));
  }
  return finish(s);
}

int rimp2_first_order(const int *nvirt_, const int *nocc_, const int *noccEOS_,
                      const int *nvirtEOS_, const int *nocctot_, const int *NBA_,
                      const double *Calpha, const double *CalphaOcc, const double *CalphaVV,
                      const double *UoccEOST, const double *UvirtT, const double *UoccT,
                      const double *UoccallT, const double *UvirtEOST, double *djik,
                      double *blad) {
  clear_error();
  RIMP2_REQ(pos(nvirt_) && pos(nocc_) && pos(noccEOS_) && pos(nvirtEOS_) && pos(nocctot_) &&
                pos(NBA_),
            "rimp2_first_order: bad dims");
  RIMP2_REQ(Calpha && CalphaOcc && CalphaVV && UoccEOST && UvirtT && UoccT && UoccallT &&
                UvirtEOST && djik && blad,
            "rimp2_first_order: null array");
  RIMP2_REQ(*nocc_ <= *nvirt_,
            "rimp2_first_order: nocc > nvirt (the CalphaVV DGEMM reads nocc rows of UvirtT)");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const int nvirt = *nvirt_, nocc = *nocc_, noccEOS = *noccEOS_, nvirtEOS = *nvirtEOS_,
            nocctot = *nocctot_, NBA = *NBA_;
  const size_t nv = nvirt, no = nocc, ne = noccEOS, ve = nvirtEOS, nt = nocctot, nb = NBA;
  DevBuf dC, dUoE, dUvT, dUoT, dUoA, dUvE;
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(dUoE, UoccEOST, no * ne, s));
  RIMP2_TRY(h2d(dUvT, UvirtT, nv * nv, s));
  RIMP2_TRY(h2d(dUoT, UoccT, no * no, s));
  RIMP2_TRY(h2d(dUoA, UoccallT, nt * nt, s));
  RIMP2_TRY(h2d(dUvE, UvirtEOST, nv * ve, s));
  const double *Ca = dC.as<double>();
  {  // djik (RIMP2.F90:177-207)
    DevBuf dOcc, c2, c3, c2b, c4, out;
    RIMP2_TRY(h2d(dOcc, CalphaOcc, nb * no * nt, s));
    RIMP2_TRY(dalloc(c2, nb * nv * ne, s));
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nvirt, noccEOS, nocc, 1.0, Ca, NBA * nvirt,
                        dUoE.as<double>(), nocc, 0.0, c2.as<double>(), NBA * nvirt, s));
    RIMP2_TRY(dalloc(c3, nb * nv * ne, s));
    RIMP2_TRY(dev_transalpha2(noccEOS, nvirt, nvirt, NBA, dUvT.as<double>(), c2.as<double>(),
                              c3.as<double>(), s));
    RIMP2_TRY(dalloc(c2b, nb * no * nt, s));
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nocc, nocctot, nocctot, 1.0, dOcc.as<double>(), NBA * nocc,
                        dUoA.as<double>(), nocctot, 0.0, c2b.as<double>(), NBA * nocc, s));
    RIMP2_TRY(dalloc(c4, nb * ne * nt, s));
    RIMP2_TRY(dev_transalpha2(nocctot, nocc, noccEOS, NBA, dUoE.as<double>(), c2b.as<double>(),
                              c4.as<double>(), s));
    RIMP2_TRY(dalloc(out, nv * ne * ne * nt, s));
    RIMP2_TRY(dev_gen4dimfo(NBA, c3.as<double>(), nvirt, noccEOS, c4.as<double>(), noccEOS, nocctot,
                            out.as<double>(), s));
    RIMP2_TRY(d2h(djik, out, nv * ne * ne * nt, s));
    RIMP2_CK(cudaStreamSynchronize(s));
  }
  {  // blad (RIMP2.F90:216-248)
    DevBuf dVV, c2, c3, c2b, c4, out;
    RIMP2_TRY(dalloc(c2, nb * nv * no, s));
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nvirt, nocc, nocc, 1.0, Ca, NBA * nvirt, dUoT.as<double>(),
                        nocc, 0.0, c2.as<double>(), NBA * nvirt, s));
    RIMP2_TRY(dalloc(c3, nb * ve * no, s));
    RIMP2_TRY(dev_transalpha2(nocc, nvirt, nvirtEOS, NBA, dUvE.as<double>(), c2.as<double>(),
                              c3.as<double>(), s));
    RIMP2_TRY(h2d(dVV, CalphaVV, nb * nv * nv, s));
    RIMP2_TRY(dalloc(c2b, nb * nv * nv, s));
    // K = ldb = nocc as in the driver's DGEMM (RIMP2.F90:232-235)
    RIMP2_TRY(dev_dgemm('N', 'N', NBA * nvirt, nvirt, nocc, 1.0, dVV.as<double>(), NBA * nvirt,
                        dUvT.as<double>(), nocc, 0.0, c2b.as<double>(), NBA * nvirt, s));
    RIMP2_TRY(dalloc(c4, nb * ve * nv, s));
    RIMP2_TRY(dev_transalpha2(nvirt, nvirt, nvirtEOS, NBA, dUvE.as<double>(), c2b.as<double>(),
                              c4.as<double>(), s));
    RIMP2_TRY(dalloc(out, ve * no * ve * nv, s));
    RIMP2_TRY(dev_gen4dimfo(NBA, c3.as<double>(), nvirtEOS, nocc, c4.as<double>(), nvirtEOS, nvirt,
                            out.as<double>(), s));
    RIMP2_TRY(d2h(blad, out, ve * no * ve * nv, s));
  }
  return finish(s);
}

int rimp2_energy_eos(const int *nvirt_, const int *nocc_, const int *noccEOS_,
                     const int *nvirtEOS_, const int *NBA_, const double *Calpha,
                     const double *EVocc, const double *EVvirt, const double *UoccEOST,
                     const double *UvirtT, const double *UoccT, const double *UvirtEOST,
                     double *Eocc, double *Evirt, const int *precision) {
  clear_error();
  RIMP2_REQ(pos(nvirt_) && pos(nocc_) && pos(noccEOS_) && pos(nvirtEOS_) && pos(NBA_),
            "rimp2_energy_eos: bad dims");
  RIMP2_REQ(Calpha && EVocc && EVvirt && UoccEOST && UvirtT && UoccT && UvirtEOST && Eocc &&
                Evirt && precision,
            "rimp2_energy_eos: null array");
  RIMP2_REQ(*precision == RIMP2_PREC_FP64 || *precision == RIMP2_PREC_SPLIT,
            "rimp2_energy_eos: precision must be 0 (FP64) or 1 (split)");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const int nvirt = *nvirt_, nocc = *nocc_, noccEOS = *noccEOS_, nvirtEOS = *nvirtEOS_,
            NBA = *NBA_;
  const size_t nv = nvirt, no = nocc, ne = noccEOS, ve = nvirtEOS, nb = NBA;
  DevBuf dC, deo, dev, dUoE, dUvT, dUoT, dUvE, Po, Pv, C1, C2, D1, Ct, Ep, Et, wk;
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(deo, EVocc, no, s));
  RIMP2_TRY(h2d(dev, EVvirt, nv, s));
  RIMP2_TRY(h2d(dUoE, UoccEOST, no * ne, s));
  RIMP2_TRY(h2d(dUvT, UvirtT, nv * nv, s));
  RIMP2_TRY(h2d(dUoT, UoccT, no * no, s));
  RIMP2_TRY(h2d(dUvE, UvirtEOST, nv * ve, s));
  const int kmax = std::max(noccEOS, nocc), vmax = std::max(nvirtEOS, nvirt);
  RIMP2_TRY(dalloc(Po, no * no, s));
  RIMP2_TRY(dalloc(Pv, nv * nv, s));
  RIMP2_TRY(dalloc(C1, nb * nv * (size_t)kmax, s));
  RIMP2_TRY(dalloc(C2, nb * nv * no, s));
  RIMP2_TRY(dalloc(D1, nb * (size_t)vmax * no, s));
  RIMP2_TRY(dalloc(Ct, nb * nv * no, s));
  RIMP2_TRY(dalloc(Ep, no * no, s));
  RIMP2_TRY(dalloc(Et, 2, s));
  RIMP2_TRY(dalloc(wk, 1, s));
  const double *Uo[2] = {dUoE.as<double>(), dUoT.as<double>()};
  const double *Uv[2] = {dUvT.as<double>(), dUvE.as<double>()};
  const int ko[2] = {noccEOS, nocc}, kv[2] = {nvirt, nvirtEOS};
  const long long MV = (long long)NBA * nvirt;
  for (int part = 0; part < 2; ++part) {
    // occupied side: C2(:,c,i) = sum_k Calpha(:,c,k) Po(k,i), Po = Uo Uo^T
    const double *c2 = C2.as<double>();
    if (2 * ko[part] <= nocc) {  // low rank: (Calpha Uo) Uo^T
      RIMP2_TRY(dev_dgemm('N', 'N', (int)MV, ko[part], nocc, 1.0, dC.as<double>(), (int)MV,
                          Uo[part], nocc, 0.0, C1.as<double>(), (int)MV, s));
      RIMP2_TRY(dev_dgemm('N', 'T', (int)MV, nocc, ko[part], 1.0, C1.as<double>(), (int)MV,
                          Uo[part], nocc, 0.0, C2.as<double>(), (int)MV, s));
    } else {
      RIMP2_TRY(dev_dgemm('N', 'T', nocc, nocc, ko[part], 1.0, Uo[part], nocc, Uo[part], nocc, 0.0,
                          Po.as<double>(), nocc, s));
      bool id = false;
      RIMP2_TRY(is_identity(Po.as<double>(), nocc, wk.as<double>(), &id, s));
      if (id)
        c2 = dC.as<double>();  // orthogonal Uo: Po = I
      else
        RIMP2_TRY(dev_dgemm('N', 'N', (int)MV, nocc, nocc, 1.0, dC.as<double>(), (int)MV,
                            Po.as<double>(), nocc, 0.0, C2.as<double>(), (int)MV, s));
    }
    // virtual side: Ct(:,a,i) = sum_c Pv(c,a) C2(:,c,i), Pv = Uv Uv^T
    const double *ct = Ct.as<double>();
    if (2 * kv[part] <= nvirt) {  // low rank: Uv (Uv^T C2)
      RIMP2_TRY(dev_transalpha2(nocc, nvirt, kv[part], NBA, Uv[part], c2, D1.as<double>(), s));
      RIMP2_TRY(dev_transalpha2_strided(nocc, kv[part], nvirt, NBA, Uv[part], nvirt, 1,
                                        D1.as<double>(), Ct.as<double>(), s));
    } else {
      RIMP2_TRY(dev_dgemm('N', 'T', nvirt, nvirt, kv[part], 1.0, Uv[part], nvirt, Uv[part], nvirt,
                          0.0, Pv.as<double>(), nvirt, s));
      bool id = false;
      RIMP2_TRY(is_identity(Pv.as<double>(), nvirt, wk.as<double>(), &id, s));
      if (id)
        ct = c2;  // orthogonal Uv: Pv = I
      else
        RIMP2_TRY(dev_transalpha2(nocc, nvirt, nvirt, NBA, Pv.as<double>(), c2, Ct.as<double>(),
                                  s));
    }
    const int ns = rimp2_split_nslices(nvirt, nocc, NBA);
    if (*precision == RIMP2_PREC_SPLIT && ns > 0)
      RIMP2_TRY(split_eos_energy(dC.as<double>(), ct, NBA, nvirt, nocc, deo.as<double>(),
                                 dev.as<double>(), Ep.as<double>(), Et.as<double>() + part,
                                 ns, s));
    else
      RIMP2_TRY(eos_energy_f64(dC.as<double>(), ct, NBA, nvirt, nocc, deo.as<double>(),
                               dev.as<double>(), Ep.as<double>(), Et.as<double>() + part, s));
  }
  double h[2];
  RIMP2_CK(cudaMemcpyAsync(h, Et.p, sizeof h, cudaMemcpyDeviceToHost, s));
  RIMP2_TRY(finish(s));
  *Eocc = h[0];
  *Evirt = h[1];
  return RIMP2_OK;
}

int rimp2_energy_dev(int nvirt, int nocc, int NBA, const double *dCalpha, const double *dEVocc,
                     const double *dEVvirt, double *dEpair, double *dEtot, double *dtamp,
                     int precision, void *stream) {
  clear_error();
  RIMP2_REQ(nvirt > 0 && nocc > 0 && NBA > 0, "rimp2_energy_dev: bad dims");
  RIMP2_REQ(dCalpha && dEVocc && dEVvirt && dEpair && dEtot, "rimp2_energy_dev: null array");
  RIMP2_REQ(precision == RIMP2_PREC_FP64 || precision == RIMP2_PREC_SPLIT,
            "rimp2_energy_dev: precision must be 0 (FP64) or 1 (split)");
  RIMP2_REQ(!(precision == RIMP2_PREC_SPLIT && dtamp),
            "rimp2_energy_dev: amplitudes are returned by the FP64 path only");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  if (precision == RIMP2_PREC_SPLIT)
    return rimp2_energy_split_dev(nvirt, nocc, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot,
                                  rimp2_split_nslices(nvirt, nocc, NBA), stream);
  PlainEnergyArgs a;
  a.Ca = dCalpha;
  a.NBA = NBA;
  a.nvirt = nvirt;
  a.nocc = nocc;
  a.eo = dEVocc;
  a.ev = dEVvirt;
  a.Epair = dEpair;
  a.Etot = dEtot;
  a.tamp = dtamp;
  a.pairs = nullptr;
  a.npairs = 0;
  return plain_energy_f64(a, s);
}

// Residual slices per element by shape bucket, chosen so that the pair and
// total energies stay within 1e-7 relative of FP64: one residual slice
// suffices once the pair sums average over enough (a,b) terms, small
// fragments get two, and fragments with fewer than 16 virtuals run in FP64
// (0): their pair energies are a handful of g^2 terms, and a near-orthogonal
// pair of columns (g ~ 1e-4 of the column norms) leaves the FP32-accumulated
// correction term with nothing to average against (1.5e-5 measured at
// nvirt = 1).  Buckets are keyed by nvirt (the (a,b) count per pair).
// Default = the table measured by rimp2_gpu_gb300/autotune.py on GB300 with a
// 2x margin on the 1e-7 target (rimp2_gpu_gb300/tuning/split_buckets.json):
// the 128-191 bucket takes one slice only on the one-CTA kernel (its four
// products: 4.2e-8 worst; the paired kernel's three: 6.1e-8), which the
// kernel table below enforces for that bucket; rimp2_set_split_buckets
// replaces it.
static std::vector<std::pair<int, int>> g_buckets = {{0, 0},   {16, 2},  {128, 1},
                                                     {192, 1}, {256, 1}, {384, 1}};
static std::mutex g_bucket_mu;

// Fragments with fewer than 64 (a,i) columns also run in FP64, whatever the
// table says: the split form's FP32 epilogue rounds every element's energy
// term (g, the reciprocal, the product) to ~2^-24, and a pair energy made of a
// handful of such terms, partly cancelling, keeps 2-5e-8 of that rounding
// (CPU emulation of the epilogue), too close to the 1e-7 bar; in FP64 such a
// fragment costs microseconds.
constexpr long long kSplitMinColumns = 64;

int rimp2_split_nslices(int nvirt, int nocc, int NBA) {
  (void)NBA;
  if ((long long)nocc * nvirt < kSplitMinColumns) return 0;
  std::lock_guard<std::mutex> lk(g_bucket_mu);
  int ns = 2;
  for (auto &b : g_buckets)
    if (nvirt >= b.first) ns = b.second;
  return ns;
}

int rimp2_set_split_buckets(int n, const int *nvirt_min, const int *nslices) {
  clear_error();
  RIMP2_REQ(n > 0 && n <= 64 && nvirt_min && nslices, "rimp2_set_split_buckets: bad table");
  std::vector<std::pair<int, int>> t;
  for (int k = 0; k < n; ++k) {
    RIMP2_REQ(nslices[k] >= 0 && nslices[k] <= 2,
              "rimp2_set_split_buckets: nslices must be 0 (FP64), 1 or 2");
    RIMP2_REQ(k == 0 || nvirt_min[k] > nvirt_min[k - 1],
              "rimp2_set_split_buckets: nvirt_min must increase");
    t.push_back({nvirt_min[k], nslices[k]});
  }
  std::lock_guard<std::mutex> lk(g_bucket_mu);
  g_buckets = t;
  return RIMP2_OK;
}

// Energy kernel of one-residual-slice fragments by shape bucket: the paired-
// CTA kernel (256-row tiles on an SM pair, three products per element pair)
// when nocc >= min_nocc and NBA >= min_nba of the bucket (largest nvirt_min
// <= nvirt), else the one-CTA kernel (128-row tiles, four products).  The
// paired kernel's per-item costs (the exchange-tile transpose, cross-CTA
// hand-offs, a dummy CTA for an odd count of i <= j) lose on short auxiliary
// spaces and few occupied orbitals.  Default = the table chosen by
// rimp2_gpu_gb300/autotune.py on GB300 (rimp2_gpu_gb300/tuning/
// split_buckets.json, "kernel_rule": fitted per bucket on isolated shapes,
// then selected among candidate tables on a mixed batch of uneven
// fragments, with the 128-191 bucket held on the one-CTA kernel for its
// accuracy); rimp2_set_split_kernel_rule replaces it.
struct KernelRule {
  int nvirt_min, min_nocc, min_nba;
};
static std::vector<KernelRule> g_krule = {{0, 16, 1024},          {16, 16, 1024},
                                           {128, 1 << 30, 1 << 30}, {192, 16, 1024},
                                           {256, 16, 1024},         {384, 12, 1024}};

}  // extern "C"

namespace rimp2 {
bool pair_kernel_for(int nocc, int nvirt, int NBA) {
  const char *e = getenv("RIMP2_PAIR_KERNEL");
  if (e && e[0] == '0') return false;
  if (e && e[0] == '1') return true;
  std::lock_guard<std::mutex> lk(g_bucket_mu);
  KernelRule r = g_krule.front();
  for (auto &b : g_krule)
    if (nvirt >= b.nvirt_min) r = b;
  return nocc >= r.min_nocc && NBA >= r.min_nba;
}
}  // namespace rimp2

extern "C" {

int rimp2_set_split_kernel_rule(int n, const int *nvirt_min, const int *min_nocc,
                                const int *min_nba) {
  clear_error();
  RIMP2_REQ(n > 0 && n <= 64 && nvirt_min && min_nocc && min_nba,
            "rimp2_set_split_kernel_rule: bad table");
  std::vector<KernelRule> t;
  for (int k = 0; k < n; ++k) {
    RIMP2_REQ(min_nocc[k] >= 1 && min_nba[k] >= 1,
              "rimp2_set_split_kernel_rule: thresholds must be positive");
    RIMP2_REQ(k == 0 || nvirt_min[k] > nvirt_min[k - 1],
              "rimp2_set_split_kernel_rule: nvirt_min must increase");
    t.push_back({nvirt_min[k], min_nocc[k], min_nba[k]});
  }
  std::lock_guard<std::mutex> lk(g_bucket_mu);
  g_krule = t;
  return RIMP2_OK;
}

int rimp2_split_kernel_for(int nvirt, int nocc, int NBA) {
  const int ns = rimp2_split_nslices(nvirt, nocc, NBA);
  if (ns == 0) return 0;
  if (ns >= 2) return 1;
  return rimp2::pair_kernel_for(nocc, nvirt, NBA) ? 2 : 1;
}

int rimp2_batch_plan_create(void **plan, int nfrag, const int *nocc, const int *nvirt,
                            const int *NBA, const double *const *dCalpha,
                            const double *const *dEVocc, const double *const *dEVvirt,
                            double *const *dEpair, double *const *dEtot, const int *nslices,
                            int use_graph, void *stream) {
  clear_error();
  RIMP2_REQ(plan, "rimp2_batch_plan_create: null plan");
  *plan = nullptr;
  RIMP2_REQ(nfrag > 0 && nocc && nvirt && NBA && dCalpha && dEVocc && dEVvirt && dEpair && dEtot,
            "rimp2_batch_plan_create: null argument");
  std::vector<int> ns(nfrag);
  for (int f = 0; f < nfrag; ++f) {
    RIMP2_REQ(nocc[f] > 0 && nvirt[f] > 0 && NBA[f] > 0 && nocc[f] < 65536,
              "rimp2_batch_plan_create: bad dims in fragment %d", f);
    RIMP2_REQ(dCalpha[f] && dEVocc[f] && dEVvirt[f] && dEpair[f] && dEtot[f],
              "rimp2_batch_plan_create: null device pointer in fragment %d", f);
    ns[f] = nslices ? nslices[f] : rimp2_split_nslices(nvirt[f], nocc[f], NBA[f]);
    RIMP2_REQ(ns[f] >= 0 && ns[f] <= 2,
              "rimp2_batch_plan_create: nslices must be 0 (FP64), 1 or 2");
  }
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  SplitPlan *P = nullptr;
  RIMP2_TRY(split_plan_create(&P, nfrag, nocc, nvirt, NBA, dCalpha, dEVocc, dEVvirt, dEpair, dEtot,
                              ns.data(), use_graph != 0, s));
  *plan = P;
  return RIMP2_OK;
}

int rimp2_batch_plan_execute(void *plan, void *stream) {
  clear_error();
  RIMP2_REQ(plan, "rimp2_batch_plan_execute: null plan");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return split_plan_execute((SplitPlan *)plan, s);
}

int rimp2_batch_plan_destroy(void *plan) {
  clear_error();
  if (plan) split_plan_destroy((SplitPlan *)plan);
  return RIMP2_OK;
}

int rimp2_energy_split_dev(int nvirt, int nocc, int NBA, const double *dCalpha,
                           const double *dEVocc, const double *dEVvirt, double *dEpair,
                           double *dEtot, int nslices, void *stream) {
  clear_error();
  RIMP2_REQ(nvirt > 0 && nocc > 0 && NBA > 0, "rimp2_energy_split_dev: bad dims");
  RIMP2_REQ(dCalpha && dEVocc && dEVvirt && dEpair && dEtot, "rimp2_energy_split_dev: null array");
  RIMP2_REQ(nslices >= 0 && nslices <= 2,
            "rimp2_energy_split_dev: nslices must be 0 (FP64), 1 or 2");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  if (nslices == 0) {  // the bucket table's FP64 tier (tiny fragments)
    PlainEnergyArgs p;
    p.Ca = dCalpha;
    p.NBA = NBA;
    p.nvirt = nvirt;
    p.nocc = nocc;
    p.eo = dEVocc;
    p.ev = dEVvirt;
    p.Epair = dEpair;
    p.Etot = dEtot;
    p.tamp = nullptr;
    p.pairs = nullptr;
    p.npairs = 0;
    return plain_energy_f64(p, s);
  }
  SplitEnergyArgs a;
  a.Ca = dCalpha;
  a.NBA = NBA;
  a.nvirt = nvirt;
  a.nocc = nocc;
  a.eo = dEVocc;
  a.ev = dEVvirt;
  a.Epair = dEpair;
  a.Etot = dEtot;
  a.nslices = nslices;
  return split_energy(a, s, nullptr);
}

int rimp2_energy(const int *nvirt, const int *nocc, const int *NBA, const double *Calpha,
                 const double *EVocc, const double *EVvirt, double *Epair, double *Etot,
                 double *tamp, const int *precision) {
  clear_error();
  RIMP2_REQ(pos(nvirt) && pos(nocc) && pos(NBA), "rimp2_energy: bad dims");
  RIMP2_REQ(Calpha && EVocc && EVvirt && Epair && Etot && precision, "rimp2_energy: null array");
  RIMP2_REQ(*precision == RIMP2_PREC_FP64 || *precision == RIMP2_PREC_SPLIT,
            "rimp2_energy: precision must be 0 (FP64) or 1 (split)");
  RIMP2_REQ(!(*precision == RIMP2_PREC_SPLIT && tamp),
            "rimp2_energy: amplitudes are returned by the FP64 path only");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nv = *nvirt, no = *nocc, nb = *NBA;
  DevBuf dC, deo, dev, dE, dT, dA;
  // the bucket table sends tiny fragments to the FP64 kernel
  if (*precision == RIMP2_PREC_SPLIT && rimp2_split_nslices(*nvirt, *nocc, *NBA) > 0) {
    // copy Calpha in occupied-index chunks overlapped with the energy work
    cudaStream_t cs = copy_stream();
    RIMP2_REQ(cs != nullptr, "rimp2_energy: copy stream unavailable");
    RIMP2_TRY(dalloc(dC, nb * nv * no, s));
    RIMP2_TRY(h2d(deo, EVocc, no, s));
    RIMP2_TRY(h2d(dev, EVvirt, nv, s));
    RIMP2_TRY(dalloc(dE, no * no, s));
    RIMP2_TRY(dalloc(dT, 1, s));
    // the copy stream must see dC allocated before it writes into it
    cudaEvent_t ready;
    RIMP2_CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    RIMP2_CK(cudaEventRecord(ready, s));
    RIMP2_CK(cudaStreamWaitEvent(cs, ready, 0));
    cudaEventDestroy(ready);
    SplitEnergyArgs a;
    a.Ca = dC.as<double>();
    a.NBA = *NBA;
    a.nvirt = *nvirt;
    a.nocc = *nocc;
    a.eo = deo.as<double>();
    a.ev = dev.as<double>();
    a.Epair = dE.as<double>();
    a.Etot = dT.as<double>();
    a.nslices = rimp2_split_nslices(*nvirt, *nocc, *NBA);
    const int chunk = std::max(1, std::min(16, (*nocc + 7) / 8));
    RIMP2_TRY(split_energy_streamed(Calpha, dC.as<double>(), a, s, cs, chunk));
    RIMP2_TRY(d2h(Epair, dE, no * no, s));
    RIMP2_TRY(d2h(Etot, dT, 1, s));
    RIMP2_CK(cudaStreamSynchronize(cs));
    return finish(s);
  }
  RIMP2_TRY(h2d(dC, Calpha, nb * nv * no, s));
  RIMP2_TRY(h2d(deo, EVocc, no, s));
  RIMP2_TRY(h2d(dev, EVvirt, nv, s));
  RIMP2_TRY(dalloc(dE, no * no, s));
  RIMP2_TRY(dalloc(dT, 1, s));
  if (tamp) RIMP2_TRY(dalloc(dA, nv * no * nv * no, s));
  RIMP2_TRY(rimp2_energy_dev(*nvirt, *nocc, *NBA, dC.as<double>(), deo.as<double>(),
                             dev.as<double>(), dE.as<double>(), dT.as<double>(),
                             tamp ? dA.as<double>() : nullptr, *precision, s));
  RIMP2_TRY(d2h(Epair, dE, no * no, s));
  RIMP2_TRY(d2h(Etot, dT, 1, s));
  if (tamp) RIMP2_TRY(d2h(tamp, dA, nv * no * nv * no, s));
  return finish(s);
}

int rimp2_energy_batched(const int *nfrag, const int *nocc, const int *nvirt, const int *NBA,
                         const double *Calpha, const long long *calpha_off, const double *EVocc,
                         const long long *eo_off, const double *EVvirt, const long long *ev_off,
                         double *Epair, const long long *epair_off, double *Etot,
                         const int *precision) {
  clear_error();
  RIMP2_REQ(nfrag && *nfrag >= 0, "rimp2_energy_batched: bad nfrag");
  RIMP2_REQ(nocc && nvirt && NBA && Calpha && calpha_off && EVocc && eo_off && EVvirt && ev_off &&
                Epair && epair_off && Etot && precision,
            "rimp2_energy_batched: null argument");
  for (int f = 0; f < *nfrag; ++f)
    RIMP2_REQ(nocc[f] > 0 && nvirt[f] > 0 && NBA[f] > 0, "rimp2_energy_batched: bad dims in %d", f);
  RIMP2_REQ(*precision == RIMP2_PREC_FP64 || *precision == RIMP2_PREC_SPLIT,
            "rimp2_energy_batched: bad precision");
  const int nf = *nfrag;
  if (nf == 0) return RIMP2_OK;
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  // one device copy of every fragment (inputs are in HBM together; the
  // split form then runs the batch as one persistent launch per kernel
  // group).  The plan is built on the destination addresses first; the
  // copies then run on the copy stream group by group, each group's kernels
  // waiting only for its own fragments (host memory pinned by the caller
  // makes the copies asynchronous, so they overlap the earlier groups)
  size_t nca = 0, neo = 0, nev = 0, nep = 0;
  for (int f = 0; f < nf; ++f) {
    nca += (size_t)NBA[f] * nvirt[f] * nocc[f];
    neo += nocc[f];
    nev += nvirt[f];
    nep += (size_t)nocc[f] * nocc[f];
  }
  DevBuf dC, deo, dev, dE, dT;
  RIMP2_TRY(dalloc(dC, nca, s));
  RIMP2_TRY(dalloc(deo, neo, s));
  RIMP2_TRY(dalloc(dev, nev, s));
  RIMP2_TRY(dalloc(dE, nep, s));
  RIMP2_TRY(dalloc(dT, nf, s));
  std::vector<const double *> pc(nf), peo(nf), pev(nf);
  std::vector<double *> pE(nf), pT(nf);
  std::vector<double *> cdst;
  std::vector<const double *> csrc;
  std::vector<size_t> ccount;
  auto copy = [&](double *d, const double *h, size_t n) {
    cdst.push_back(d);
    csrc.push_back(h);
    ccount.push_back(n);
  };
  size_t oc = 0, oo = 0, ov = 0, oe = 0;
  for (int f = 0; f < nf; ++f) {
    const size_t n = (size_t)NBA[f] * nvirt[f] * nocc[f];
    copy(dC.as<double>() + oc, Calpha + calpha_off[f], n);
    copy(deo.as<double>() + oo, EVocc + eo_off[f], (size_t)nocc[f]);
    copy(dev.as<double>() + ov, EVvirt + ev_off[f], (size_t)nvirt[f]);
    pc[f] = dC.as<double>() + oc;
    peo[f] = deo.as<double>() + oo;
    pev[f] = dev.as<double>() + ov;
    pE[f] = dE.as<double>() + oe;
    pT[f] = dT.as<double>() + f;
    oc += n;
    oo += nocc[f];
    ov += nvirt[f];
    oe += (size_t)nocc[f] * nocc[f];
  }
  {
    // split: per-fragment slice count from the bucket table, and the
    // paired-kernel fragments (the largest launch group by volume) divided
    // between NPART plans by Calpha volume, so that each part's persistent
    // launch starts while the later parts are still being copied; FP64:
    // every fragment in one plain persistent launch
    constexpr int NPART = 4;
    const bool split = *precision == RIMP2_PREC_SPLIT;
    std::vector<int> part(nf, 0);
    if (split) {
      size_t tot = 0, acc = 0;
      std::vector<char> paired(nf, 0);
      for (int f = 0; f < nf; ++f)
        if (rimp2_split_kernel_for(nvirt[f], nocc[f], NBA[f]) == 2) {
          paired[f] = 1;
          tot += (size_t)NBA[f] * nvirt[f] * nocc[f];
        }
      for (int f = 0; f < nf; ++f)
        if (paired[f]) {
          part[f] = (int)std::min<size_t>(NPART - 1, acc * NPART / tot);
          acc += (size_t)NBA[f] * nvirt[f] * nocc[f];
        }
    }
    // one copy stream: the transfer runs at the host link's rate (~130 GB/s
    // measured; copies spread over four streams made the call slower, 234
    // against 215 ms for 27.9 GB)
    cudaStream_t cs = copy_stream();
    if (!cs) {
      set_error("copy stream creation failed");
      return RIMP2_ERR_CUDA;
    }
    void *plans[NPART] = {};
    std::vector<double *> pd[NPART];
    std::vector<const double *> ps[NPART];
    std::vector<size_t> pn[NPART];
    int rc = RIMP2_OK;
    for (int p = 0; p < NPART && rc == RIMP2_OK; ++p) {
      std::vector<int> o, v, b;
      std::vector<const double *> c, e1, e2;
      std::vector<double *> E, T;
      for (int f = 0; f < nf; ++f) {
        if (part[f] != p) continue;
        o.push_back(nocc[f]);
        v.push_back(nvirt[f]);
        b.push_back(NBA[f]);
        c.push_back(pc[f]);
        e1.push_back(peo[f]);
        e2.push_back(pev[f]);
        E.push_back(pE[f]);
        T.push_back(pT[f]);
        for (int q = 3 * f; q < 3 * f + 3; ++q) {  // Calpha, EVocc, EVvirt of fragment f
          pd[p].push_back(cdst[q]);
          ps[p].push_back(csrc[q]);
          pn[p].push_back(ccount[q]);
        }
      }
      if (o.empty()) continue;
      std::vector<int> zeros(o.size(), 0);
      rc = rimp2_batch_plan_create(&plans[p], (int)o.size(), o.data(), v.data(), b.data(), c.data(),
                                   e1.data(), e2.data(), E.data(), T.data(),
                                   split ? nullptr : zeros.data(), 0, s);
    }
    // a later plan's copies queue behind the earlier plans' on the copy
    // stream, which waited for the allocations once
    bool waited = false;
    for (int p = 0; p < NPART && rc == RIMP2_OK; ++p)
      if (plans[p]) {
        rc = split_plan_execute_host((SplitPlan *)plans[p], s, &cs, 1, (int)pd[p].size(),
                                     pd[p].data(), ps[p].data(), pn[p].data(), !waited);
        waited = true;
      }
    // after a failure some copies may still be in flight on the copy stream,
    // not ordered before the buffers' release on s: let them finish first
    if (rc != RIMP2_OK) cudaStreamSynchronize(cs);
    for (auto pl : plans)  // keeps the error message of a failed execute
      if (pl) split_plan_destroy((SplitPlan *)pl);
    RIMP2_TRY(rc);
  }
  oe = 0;
  for (int f = 0; f < nf; ++f) {
    RIMP2_CK(cudaMemcpyAsync(Epair + epair_off[f], dE.as<double>() + oe,
                             (size_t)nocc[f] * nocc[f] * 8, cudaMemcpyDeviceToHost, s));
    oe += (size_t)nocc[f] * nocc[f];
  }
  RIMP2_CK(cudaMemcpyAsync(Etot, dT.p, (size_t)nf * 8, cudaMemcpyDeviceToHost, s));
  return finish(s);
}

}  // extern "C"
