// common.cuh -- shared definitions of the rimp2_gpu_gb300 CUDA library.
//
// One process, one GPU, one library-owned CUDA stream (or a stream the caller
// hands over).  Every C-ABI entry point returns an int status and never
// aborts; the message of the last failure on the calling thread is kept for
// rimp2_last_error_string().
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>

#include "../../include/rimp2_gpu.h"

namespace rimp2 {

// ---- status / error handling ------------------------------------------------
void set_error(const char *fmt, ...);
void clear_error();
cudaStream_t current_stream();
int ensure_device();  // RIMP2_OK or an error status (message set)
int *device_error_word();  // persistent device int that kernels set on a failed bounded wait
int collect_device_error(cudaStream_t s);  // sync s, read + clear the word, map to a status
// optional per-phase event timing of the split path (ms of the last call)
bool timing_enabled();
void record_timing(int slot, float ms);

#define RIMP2_CK(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      ::rimp2::set_error("%s:%d %s -> %s", __FILE__, __LINE__, #call,               \
                         cudaGetErrorString(e_));                                   \
      return e_ == cudaErrorMemoryAllocation ? RIMP2_ERR_NOMEM : RIMP2_ERR_CUDA;    \
    }                                                                               \
  } while (0)

#define RIMP2_REQ(cond, ...)                  \
  do {                                        \
    if (!(cond)) {                            \
      ::rimp2::set_error(__VA_ARGS__);        \
      return RIMP2_ERR_ARG;                   \
    }                                         \
  } while (0)

#define RIMP2_TRY(expr)          \
  do {                           \
    int s_ = (expr);             \
    if (s_ != RIMP2_OK) return s_; \
  } while (0)

// Stream-ordered device buffer (memory pool backed); freed on scope exit.
struct DevBuf {
  void *p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  int alloc(size_t bytes, cudaStream_t st);
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

// Host fault injection for failure-path tests: RIMP2_FAULT_INJECT=alloc makes
// the next device allocation report out-of-memory, =launch makes the next
// kernel-launch check report a launch failure.  Nothing touches the GPU.
bool inject_fault(const char *what);

// ---- FP64 DMMA kernels (fp64_kernels.cu) -------------------------------------
struct GemmDesc {
  int M, N, K;
  double alpha, beta;
  const double *A;
  long long sAm, sAk, sAb0, sAb1;  // element strides: row m, reduction k, batch dims
  const double *B;
  long long sBk, sBn, sBb0, sBb1;
  double *C;
  long long sCm, sCn, sCb0, sCb1;
  int nb0, nb1;  // batch extents (nb0 fastest)
  // optional epilogue: divide by (eo[i]+eo[j]-ev[n]-ev[m]) where (i,j) come
  // from the two batch indices (used by the toccA/tvirtA g/D step)
  const double *eo, *ev;
  int denom;  // 0 none, 1 batch=(i,j) row=a col=b
  int lower;  // 1: only output tiles touching the lower triangle (m >= n) are computed
};
int launch_gemm_f64(const GemmDesc &g, cudaStream_t s);

struct PlainEnergyArgs {
  const double *Ca;  // Calpha(NBA, nvirt, nocc)
  int NBA, nvirt, nocc;
  const double *eo, *ev;
  double *Epair;     // nocc*nocc (device)
  double *Etot;      // 1 (device)
  double *tamp;      // optional (nvirt, nocc, nvirt, nocc) (device) or null
  const int *pairs;  // optional (i<=j) pairs list, device, 2*npairs; null = all
  int npairs;
};
int plain_energy_f64(const PlainEnergyArgs &a, cudaStream_t s);
int probe_fp64_peak(double *tflops, cudaStream_t s);
void plain_energy_scratch_sizes(int nvirt, int nocc, long long *npairs, long long *nitems);
int plain_energy_f64_scratch(const PlainEnergyArgs &a, int *pairs_scratch, double *part_scratch,
                             cudaStream_t s);
int preload_plain_scratch_kernels();
// Loads the allocation-free entry point's scratch array and kernels onto the
// current device (ensure_device calls it on the library's first use).
int noalloc_preload();
// Fused local-orbital energy from Calpha and its projected copy Ct (FP64).
int eos_energy_f64(const double *Ca, const double *Ct, int NBA, int nvirt, int nocc,
                   const double *eo, const double *ev, double *Epair, double *Etot,
                   cudaStream_t s);
// Batched plain FP64 energies: every fragment's (pair, 64x64 tile pair) items
// in one persistent launch, then per-fragment compensated reductions.
struct PlainFrag {
  const double *Ca, *eo, *ev;
  double *Epair, *Etot;
  int nocc, nvirt, NBA, ntp;
  int pair_base;        // first global pair index
  long long item_base;  // first work item
};
struct PlainPlan;
int plain_plan_create(PlainPlan **out, int nfrag, const PlainFrag *frags, cudaStream_t s);
int plain_plan_record(PlainPlan *P, cudaStream_t s);  // no sync, no allocation
int plain_plan_launches(const PlainPlan *P);
void plain_plan_destroy(PlainPlan *P);

// ---- split-precision tcgen05 path (split_kernels.cu) ---------------------------
struct SplitEnergyArgs {
  const double *Ca;
  int NBA, nvirt, nocc;
  const double *eo, *ev;
  double *Epair, *Etot;
  int nslices;  // residual slices per element (1 or 2)
};
int split_energy(const SplitEnergyArgs &a, cudaStream_t s, float *ms_kernel);
// local-orbital fragment energy (Calpha and its projected copy Ct), split form
int split_eos_energy(const double *Ca, const double *Ct, int NBA, int nvirt, int nocc,
                     const double *eo, const double *ev, double *Epair, double *Etot,
                     int nslices, cudaStream_t s);
struct SplitPlan;
int split_plan_create(SplitPlan **out, int nfrag, const int *nocc, const int *nvirt, const int *NBA,
                      const double *const *Ca, const double *const *eo, const double *const *ev,
                      double *const *Epair, double *const *Etot, const int *nslices, bool graph,
                      cudaStream_t s);
int split_plan_execute(SplitPlan *P, cudaStream_t s);
int split_plan_execute_host(SplitPlan *P, cudaStream_t s, const cudaStream_t *cs, int ncs,
                            int ncopy, double *const *dst, const double *const *src,
                            const size_t *count, bool wait_alloc = true);
void split_plan_destroy(SplitPlan *P);
int bounded_wait_selftest(long long budget_cycles, cudaStream_t s);
int rcp_denom_selftest(int n, const float *d, float *r, float *ref, cudaStream_t s);
int split_energy_streamed(const double *hCa, double *dCa, const SplitEnergyArgs &a,
                          cudaStream_t s, cudaStream_t copy_s, int chunk_occ);
cudaStream_t copy_stream();
cudaStream_t slice_stream();  // the streamed host path's slicing
// K-major FP16 slices of a set of rows (split GEMM operand)
struct SlicedOp {
  int nsl = 2, nks = 0;
  long long rows_per_group = 0, ncol = 0, R = 0;
  DevBuf slices, inv, desc;
};
// rows = columns of a column-major array: group g, row r at src + K*(r + nrows*g)
int sliced_cols(SlicedOp &op, const double *src, int K, int nrows, int ngroups, int nsl,
                cudaStream_t s);
// half[i][alpha][mu] = sum_nu ao(alpha,mu,nu) Cmo(nu,i) in one fused pass over
// the AO tensor; *handled = false when nocc is beyond the fused kernel
int ao_half_fused(const double *ao, int NBA, int nbas, const double *Cmo, int nocc, double *half,
                  cudaStream_t s, bool *handled);
// rows m' = mu + nbas*alpha of (alpha|mu nu) over K = nu
int sliced_ao(SlicedOp &op, const double *ao, int NBA, int nbas, int nsl, cudaStream_t s);
// out[b*sOb + m*sOm + n*sOn] = sum_k A[a_row0 + b*a_bstride + m][k] * B[b_row0 + b*b_bstride + n][k]
int split_gemm(const SlicedOp &A, long long a_row0, long long a_bstride, const SlicedOp &B,
               long long b_row0, long long b_bstride, int M, int N, int nbatch, double *out,
               long long sOm, long long sOn, long long sOb, cudaStream_t s);
bool split_supported();
// Energy kernel of a one-residual-slice fragment: true = paired-CTA kernel
// (kernel-rule table of capi.cu; RIMP2_PAIR_KERNEL=0/1 overrides it)
bool pair_kernel_for(int nocc, int nvirt, int NBA);

}  // namespace rimp2
