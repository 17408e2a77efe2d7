// split_kernels.cu -- split-precision RI-MP2 energy on the tcgen05 tensor cores.
//
// Numerics (Ozaki-style integer slices carried in FP16):
//   For every column c=(a,i) of Calpha(:,a,i) a power-of-two scale s_c is
//   chosen so that |C*s_c| <= 2047.5 and ||round(C*s_c)||_2 <= 2^12.  Then
//     C*s_c = S0 + R1 (+ R2)
//   with S0 = round(C*s_c) an integer in [-2048,2048] (exact in FP16) and R1, R2
//   the FP16-rounded residuals.  The alpha contraction of two columns is
//     g*s_a*s_b = sum S0a S0b  +  sum (S0a R1b + R1a S0b + R1a R1b [+ S0a R2b + R2a S0b])
//   The first sum (accumulator L0) is a sum of integers whose every partial
//   sum is bounded by ||S0a|| ||S0b|| <= 2^24 (Cauchy-Schwarz), so the FP32
//   tensor-core accumulation is EXACT whatever its internal rounding mode.
//   The correction terms (accumulator L1) are ~2^-8 of g and uncorrelated
//   with it, so their FP32 rounding does not bias the energy.
//   The epilogue forms g in FP32, the denominator from hi/lo float pairs of
//   the FP64 orbital energies, and accumulates e_ij in FP32 per thread and
//   FP64 across threads; pair and total energies are reduced in FP64 with
//   compensation.
//
// Kernel layout (one persistent CTA per SM, 576 threads):
//   warp 0       TMA producer (128x64 FP16 boxes, 128B swizzle) and the
//                device-side work queue (atomic counter, 4-deep item ring)
//   warp 1       TMEM owner + single-thread tcgen05.mma issuer
//   warps 2..17  epilogue, four warps per TMEM lane quadrant (32 accumulator
//                columns each): tcgen05.ld, denominators, energy terms
//   Work item = (fragment, pair i<=j, tile pair A<=B): T1 = G_ij[A,B] =
//   C_iA^T C_jB and T2 = G_ji[A,B] = C_jA^T C_iB, each with L0/L1
//   accumulators in TMEM (4 x 128 columns = all 512).  The exchange integral
//   g_ij(b,a) = T2[a,b] therefore lives in the same TMEM lane/column as
//   g_ij(a,b) = T1[a,b], and no four-index quantity is ever written to
//   memory.  T1 is read out and released first, so the next item's T1 MMAs
//   overlap this item's T2 phase; diagonal tile pairs take T2 = T1^T through
//   shared memory.
// A one-residual-slice fragment with enough occupied orbitals and a long
// enough auxiliary space (the measured kernel table of capi.cu) runs instead
// on split_pair_kernel: clusters of two CTAs issuing cta_group::2 MMAs over
// two occupied pairs that share their B operand, with a third slice plane
// V = fp16(C*s) that folds R1a S0b + R1a R1b into R1a V (three products per
// element pair, a per-column correction removing the same-column bias).
// Every wait on an mbarrier is bounded by a clock budget; on expiry the
// kernel records an error code, drains its own copies and MMAs, frees TMEM
// and returns, and the host reports RIMP2_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace rimp2 {

void count_launch(int n);
void note_split_kernel(int k);  // 1 one-CTA, 2 paired-CTA
__global__ void pair_reduce_kernel(const double *__restrict__ part, int nper, const int *pairs,
                                   int npairs, int nocc, double *Epair);
__global__ void total_reduce_kernel(const double *Epair, int nocc, double *Etot);
__global__ void make_pairs_kernel(int nocc, int *pairs);

namespace {

constexpr int TILE = 128;      // a/b tile edge (MMA M and N)
constexpr int KSTEP = 64;      // K per stage (one 128-byte swizzle row of FP16)
constexpr int PANEL_BYTES = TILE * KSTEP * 2;  // 16 KB
constexpr int NTHREADS = 320;  // producer warp, MMA warp, 8 epilogue warps
constexpr long long WAIT_BUDGET = 4000000000LL;  // ~2 s of SM clock per wait
// split_batch_kernel: producer warp, MMA warp and 16 epilogue warps (four per
// TMEM lane quadrant, 32 accumulator columns each; the launch bounds give
// them 96 registers).  On short auxiliary spaces a work item is bounded by
// its epilogue and hand-offs, not by its MMAs; 16 warps instead of 8 took
// 5-7% off such items (nocc=64 nvirt=512 NBA=256) and left long ones as
// they were.
constexpr int BATCH_EPI = 16;
constexpr int BATCH_THREADS = 64 + 32 * BATCH_EPI;

// --------------------------------------------------------------------------
// small PTX helpers
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false (and raises the CTA abort flag and the global
// error word) if the phase does not complete within the clock budget or if
// another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code, long long budget = WAIT_BUDGET) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > budget) {
      *abort_flag = 1;
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

// OR of a predicate over the 256 epilogue threads (named barrier 1).  The
// epilogue warps leave their loop together on a failed bounded wait, so that
// none is left waiting at a later named barrier for a warp that has gone.
__device__ __forceinline__ bool epi_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 1, 256, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}

// the same over the 512 epilogue threads of split_batch_kernel
__device__ __forceinline__ bool epi_any512(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 1, 512, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"((uint64_t)map), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// K-major operand tile of 128 rows x 64 FP16 (128-byte rows), 128B swizzle,
// 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)(16 >> 4) << 16;                  // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset: 8-row group pitch
  d |= (uint64_t)1 << 46;                          // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                          // swizzle: 128B
  return d;
}

// Instruction descriptor: kind::f16, A=B=F16, D=F32, K-major A and B, M=128, N=128
constexpr uint32_t IDESC = (1u << 4)            // D format F32
                           | (0u << 7)          // A format F16
                           | (0u << 10)         // B format F16
                           | ((uint32_t)(TILE >> 3) << 17)   // N >> 3
                           | ((uint32_t)(TILE >> 4) << 24);  // M >> 4

// the same with N = 256 (two stacked 128-row B panels)
constexpr uint32_t IDESC_N256 = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(TILE >> 4) << 24);

// kind::f16, F16 operands, F32 accumulator, K-major, M rows, N columns
// (M = 128: N a multiple of 16 up to 256)
__host__ __device__ constexpr uint32_t idesc_mn(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_f16_id(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                           uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// Reciprocal of an energy denominator (never zero or subnormal here): the
// hardware approximation (PTX rcp.approx.ftz.f32, about one ulp) refined by
// one Newton-Raphson step r' = r + r (1 - d r), whose residual 1 - d r is
// exact in one FMA; the result is within about half an ulp, so a fragment
// whose denominators are all equal does not accumulate a one-sided error.
__device__ __forceinline__ float rcp_denom(float d) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
  const float e = fmaf(-d, r, 1.0f);
  return fmaf(r, e, r);
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void decode_tri(int q, int &A, int &B) {
  int b = (int)((sqrtf(8.0f * q + 1.0f) - 1.0f) * 0.5f);
  while ((b + 1) * (b + 2) / 2 <= q) ++b;
  while (b * (b + 1) / 2 > q) --b;
  B = b;
  A = q - b * (b + 1) / 2;
}

// --------------------------------------------------------------------------
// slicing kernel: Calpha (FP64) -> FP16 slices + per-column inverse scales
// --------------------------------------------------------------------------
// slices layout: [slice][col][Kpad] FP16, col = a + nvpad*i (padded columns
// and padded K are zero); inv_scale[col] = 2^-e.
//
// GB300 runs FP64 arithmetic at a small fraction of its FP32 rate, so the
// per-element work here avoids the FP64 pipe: the scaled value's integer
// part and remainder come from the mantissa bits by integer arithmetic
// (split_int below), the remainder is then rounded to FP16 slices in FP32.
// Only the per-column scale choice uses FP64, in one thread per column.
// One fragment of a batch: sizes, where its data lives, where its slices,
// scales, work items and pair energies go.
struct FragDesc {
  int nocc, nvirt, nvpad, NBA;
  int nks;              // K chunks of 64
  int ntp;              // tile pairs A<=B
  int ncol;             // nocc * nvpad
  int eo_off, ev_off;   // into eo2 / ev2
  int pair_base;        // first global pair index
  long long row_base;   // first 64-wide slice row (per slice plane)
  long long col_base;   // first inverse-scale index
  long long item_base;  // first work item
  long long pitem_base; // first pair item (paired-CTA kernel)
  const double *Ca, *eo, *ev;
  double *Epair, *Etot;
};

__device__ __forceinline__ int find_frag_item(const FragDesc *fr, int nfrag, long long x) {
  int lo = 0, hi = nfrag - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (fr[mid].item_base <= x)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void decode_pair(int p, int &i, int &j) {
  int jj = (int)((sqrtf(8.0f * p + 1.0f) - 1.0f) * 0.5f);
  while ((jj + 1) * (jj + 2) / 2 <= p) ++jj;
  while (jj * (jj + 1) / 2 > p) --jj;
  j = jj;
  i = p - jj * (jj + 1) / 2;
}

// Per-element arithmetic of the slicing kernels in 32/64-bit integer
// operations on the FP64 bit pattern: GB300's FP64 pipe is far too slow for
// per-element work, and assembling floats with ldexpf costs several times
// more instructions (the slicing kernels are issue-bound, ncu).
//
// |v| truncated to float (mantissa cut to 24 bits), for a column's sum of
// squares: the exponent is rebiased in place; values below the float range
// count as 0, values above it as FLT_MAX.
__device__ __forceinline__ float abs_trunc_f32(unsigned long long mag) {
  const unsigned int ed = (unsigned int)(mag >> 52);
  if (ed < 897u) return 0.0f;
  if (ed > 1150u) return 3.4028234663852886e38f;
  return __uint_as_float((unsigned int)((mag >> 29) - (896ull << 23)));
}

// float -> double by moving bits (GB300 runs the F2F conversion on its slow
// FP64 pipe): normal floats and zero; a subnormal float becomes zero.
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t ex = (u >> 23) & 0xFFu;
  const uint32_t hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u >> 3) & 0xFFFFFu);
  const uint32_t lo = u << 29;
  return ex == 0 ? 0.0 : __hiloint2double((int)hi, (int)lo);
}

// v * p for p = 2^k (a normal float) by adding k to v's exponent field:
// exact; zero stays zero, a result below the normal range becomes zero.
__device__ __forceinline__ double scale_pow2(double v, float p) {
  const int k = (int)((__float_as_uint(p) >> 23) & 0xFFu) - 127;
  const long long bits = __double_as_longlong(v);
  const int ev = (int)((bits >> 52) & 0x7FF);
  if (ev == 0) return v;
  if (ev + k <= 0) return 0.0;
  return __longlong_as_double(bits + ((long long)k << 52));
}

// Split of a double x with |x 2^e| < 2^22 into q (an integer, rounded half to
// even; |q| <= 512 for the AO chunks, <= 2048 for Calpha columns) and r ~ x 2^e - q in FP32 arithmetic only (GB300's
// FP64 pipe is a small fraction of the FP32 one): v = |x| 2^e is the float
// f_hi holding the top 24 significant bits of x (exponent and fraction bits
// moved into place, no rounding) plus f_lo holding the next 23 bits (a 23-bit
// integer formed with the 2^23 magic constant, times a power of two);
// q = round(f_hi) with the 1.5 * 2^23 constant, r = (f_hi - q) + f_lo, where
// f_hi - q is exact and the sum rounds once (2^-25 of |r|).  Values below
// 2^-40 of the scaled unit, zeros and subnormals give q = r = 0.  The sign
// of x goes onto both.  Equal to split_int's results to within its rounding
// of r; tests/test_split_numerics_cpu.py restates these float operations and
// checks them against exact rational arithmetic.
__device__ __forceinline__ void split_f32(double x, int e, float &q, float &r) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t sgn = hi & 0x80000000u;
  const int ed = (int)((hi >> 20) & 0x7FFu);
  const int E = ed - 1023 + e;  // |x| 2^e = 1.f 2^E
  const bool live = ed != 0 && E >= -40;
  const int Ec = live ? E : 0;
  const uint32_t frac23 = (__funnelshift_l(lo, hi, 3)) & 0x7FFFFFu;
  const float fhi = __uint_as_float(((uint32_t)(Ec + 127) << 23) | frac23);
  const float lo23 = __uint_as_float(0x4B000000u | ((lo >> 6) & 0x7FFFFFu)) - 8388608.0f;
  const float flo = lo23 * __uint_as_float((uint32_t)(Ec - 46 + 127) << 23);
  const float qm = (fhi + 12582912.0f) - 12582912.0f;
  const float rm = (fhi - qm) + flo;
  q = live ? __uint_as_float(__float_as_uint(qm) | sgn) : 0.0f;
  r = live ? __uint_as_float(__float_as_uint(rm) ^ sgn) : 0.0f;
}

// x = |v| 2^e split into q = rint(x) (round half to even; |q| <= 2048 by the
// choice of e) and the remainder r = x - q, from A = floor(x 2^32): the
// integer part and the 32 bits below it of the 53-bit mantissa.  r is exact
// to 2^-31 absolute, far below what the FP16 residual slices keep (R1 rounds
// r to 11 bits, R2 the rest to 11 more, ~2^-24 absolute).  The sign of v is
// applied to both.
__device__ __forceinline__ void split_int(unsigned long long b, int e, float &q, float &r) {
  const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
  const int ed = (int)(mag >> 52);
  const int sh = 1075 - 32 - ed - e;  // A = M >> sh, M the mantissa with its leading 1
  unsigned long long A = 0;
  if (ed != 0 && sh < 64) {
    const unsigned long long M = (mag & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
    A = sh >= 0 ? (M >> sh) : (M << (-sh));
  }
  const unsigned long long qi = (A + 0x7FFFFFFFull + ((A >> 32) & 1ull)) >> 32;
  const long long fr = (long long)A - (long long)(qi << 32);  // in [-2^31, 2^31]
  float qf = (float)(unsigned int)qi;
  float rf = (float)(int)(fr >> 1) * 4.656612873077393e-10f;  // 2^-31
  if (b >> 63) {
    qf = -qf;
    rf = -rf;
  }
  q = qf;
  r = rf;
}

// Power-of-two scale exponent of a column from its largest magnitude (bits)
// and its FP32 sum of squares: |C 2^e| <= 2047.5 and ||C 2^e||_2 below 2^12
// with room for the rounding of NBA values.  Integer and FP32 arithmetic only
// (GB300's FP64 pipe is a small fraction of its FP32 rate, and the FP64
// sqrt/div/log2 of this choice, once per column, bounded the slicing
// kernels): with max |C| = m 2^E (m in [1, 2)), 2047.5 / m lies in
// (1023.75, 2047.5], so the magnitude bound allows e = 10 - E when m <=
// 2047.5 / 1024 = 2 - 2^-11 (fraction bits <= 0xFFE00 << 32) and 9 - E
// otherwise; the norm bound takes the binary exponent of the FP32 ratio,
// correctly rounded operations with a 2^-20 margin (float
// truncation of the squares underestimates ||C||^2 by < 2^-21 relative; the
// caller's exact integer check of ||S0||^2 keeps the exactness either way).
// Clamped to [-100, 100]; 0 for an all-zero column.
__device__ __forceinline__ int col_scale_exponent(unsigned long long mxb, float ss, int NBA) {
  if (mxb == 0) return 0;
  const int ed = (int)(mxb >> 52);
  if (ed == 0) return 100;  // largest value subnormal
  const int e1 = ((mxb & 0xFFFFFFFFFFFFFull) <= (0xFFE00ull << 32) ? 10 : 9) - (ed - 1023);
  int e2 = 127;
  if (ss > 0.0f) {
    const float r = (4096.0f - 0.5f * sqrtf((float)NBA)) / sqrtf(ss) * 0.99999905f;
    e2 = (int)((__float_as_uint(r) >> 23) & 0xFFu) - 127;  // floor(log2 r) for r normal
  }
  return max(-100, min(100, min(e1, e2)));
}

// Slices of every fragment: slice plane s, fragment f, K chunk kc, column c
// live at row (row_base_f + kc*ncol_f + c) of 64 FP16, i.e. one 2D-boxable
// K-chunk-major layout shared by all fragments (one tensor map per batch).
// grid.y = fragment, one warp per column.  At most 40 registers a thread, so
// that a 256-thread block fits in the registers a persistent energy kernel
// leaves free on its SM: in a batch graph the next group's slicing runs
// beside the current group's energy kernel.  (A single-pass form holding the
// column in registers was measured slower: a 12 KB column took ~40 KB of
// register file, leaving too few columns in flight per SM.)
__global__ void __launch_bounds__(256, 6)
    slice_batch_kernel(const FragDesc *__restrict__ fr, int nsl, long long plane,
                                   __half *__restrict__ slices, float *__restrict__ inv_scale,
                                   int col0, int col1, int vplane = 0,
                                   float *__restrict__ dcorr = nullptr) {
  // columns [col0, min(col1, ncol)) of each fragment
  const FragDesc &F = fr[blockIdx.y];
  const int col = col0 + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= F.ncol || col >= col1) return;
  const int a = col % F.nvpad, i = col / F.nvpad;
  const int Kpad = F.nks * 64;
  const __half hz = __float2half_rn(0.0f);
  __half *out = slices + (size_t)(F.row_base + col) * 64;
  const size_t kstride = (size_t)F.ncol * 64;  // next K chunk of the same column
  if (a >= F.nvirt) {
    for (int k0 = 4 * lane; k0 < Kpad; k0 += 128) {
      const size_t o = (size_t)(k0 >> 6) * kstride + (k0 & 63);
      for (int sl = 0; sl < nsl + vplane; ++sl)
        *reinterpret_cast<uint2 *>(out + sl * plane + o) = make_uint2(0u, 0u);
    }
    if (lane == 0) {
      inv_scale[F.col_base + col] = 1.0f;
      if (vplane) dcorr[F.col_base + col] = 0.0f;
    }
    return;
  }
  const int NBA = F.NBA;
  const double *c = F.Ca + ((size_t)i * F.nvirt + a) * NBA;
  unsigned long long mxb = 0;
  float ss = 0.0f;
  // four independent loads in flight per lane (the pass is latency-bound)
  for (int k0 = lane; k0 < NBA; k0 += 128) {
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = (k0 + 32 * u < NBA) ? c[k0 + 32 * u] : 0.0;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const unsigned long long mag =
          (unsigned long long)__double_as_longlong(v[u]) & 0x7FFFFFFFFFFFFFFFull;
      mxb = mag > mxb ? mag : mxb;
      const float f = abs_trunc_f32(mag);
      ss = fmaf(f, f, ss);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, mxb, o);
    mxb = other > mxb ? other : mxb;
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
  }
  int e = lane == 0 ? col_scale_exponent(mxb, ss, NBA) : 0;
  e = __shfl_sync(0xffffffffu, e, 0);
  if (vplane && lane == 0) dcorr[F.col_base + col] = 0.0f;
  for (int attempt = 0; attempt < 64; ++attempt) {
    long long n2 = 0;  // sum of S0^2 (integers; <= 2^24 is the test)
    float dsum = 0.0f;  // sum of R1 (V - S0 - R1) (V plane only)
    // four consecutive K values per lane (one 8-byte store per plane; a
    // 64-wide K chunk holds 16 lanes' groups); values beyond NBA are zeros
    for (int k0 = 4 * lane; k0 < Kpad; k0 += 128) {
      double v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = (k0 + u < NBA) ? c[k0 + u] : 0.0;
      __align__(8) __half h0[4], h1[4], h2[4], hv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float q, r;
        split_f32(v[u], e, q, r);  // zeros give q = r = 0
        h0[u] = __float2half_rn(q);  // integer |q| <= 2048: exact in FP16
        h1[u] = __float2half_rn(r);
        h2[u] = __float2half_rn(r - __half2float(h1[u]));
        // |q| < 2^23: its integer value from the 2^23 magic constant
        const int qi = __float_as_int(fabsf(q) + 8388608.0f) - 0x4B000000;
        n2 += qi * qi;  // |q| <= 2048: q^2 fits an int
        if (vplane) {
          // V = C*s in FP16; its rounding error against S0 + R1 is exact in FP32
          hv[u] = __float2half_rn(q + r);
          const float r1 = __half2float(h1[u]);
          dsum = fmaf(r1, (__half2float(hv[u]) - q) - r1, dsum);
        }
      }
      const size_t o = (size_t)(k0 >> 6) * kstride + (k0 & 63);
      *reinterpret_cast<uint2 *>(out + o) = *reinterpret_cast<const uint2 *>(h0);
      if (nsl > 1) *reinterpret_cast<uint2 *>(out + plane + o) = *reinterpret_cast<const uint2 *>(h1);
      if (nsl > 2)
        *reinterpret_cast<uint2 *>(out + 2 * plane + o) = *reinterpret_cast<const uint2 *>(h2);
      if (vplane)
        *reinterpret_cast<uint2 *>(out + nsl * plane + o) = *reinterpret_cast<const uint2 *>(hv);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
    if (n2 <= 16777216LL) {  // ||S0||^2 <= 2^24: L0 accumulation exact
      if (vplane) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        if (lane == 0) dcorr[F.col_base + col] = dsum;
      }
      break;
    }
    --e;
  }
  if (lane == 0) inv_scale[F.col_base + col] = ldexpf(1.0f, -e);
}

// orbital energies as hi/lo float pairs (padded virtuals get a large value so
// their denominators stay finite; their g is exactly zero). grid.y = fragment
__global__ void eps_batch_kernel(const FragDesc *__restrict__ fr, float2 *eo2, float2 *ev2) {
  const FragDesc &F = fr[blockIdx.y];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < F.nocc) {
    const double v = F.eo[t];
    const float h = (float)v;
    eo2[F.eo_off + t] = make_float2(h, (float)(v - (double)h));
  }
  if (t < F.nvpad) {
    const double v = t < F.nvirt ? F.ev[t] : 1000.0;
    const float h = (float)v;
    ev2[F.ev_off + t] = make_float2(h, (float)(v - (double)h));
  }
}

// Work items in queue order: fragments are enumerated heaviest first (the
// host orders the descriptors by K length), pairs j-major, tile pairs
// B-major.  item = {fragment, i | j<<16, tA | tB<<16, item id}.
__global__ void build_items_kernel(const FragDesc *__restrict__ fr, int nfrag, long long nitems,
                                   int4 *__restrict__ items) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nitems) return;
  const int f = find_frag_item(fr, nfrag, t);
  const FragDesc &F = fr[f];
  const long long loc = t - F.item_base;
  const int p = (int)(loc / F.ntp), q = (int)(loc % F.ntp);
  int i, j, tA, tB;
  decode_pair(p, i, j);
  decode_tri(q, tA, tB);
  items[t] = make_int4(f, i | (j << 16), tA | (tB << 16), (int)t);
}

struct BatchParams {
  const FragDesc *frags;
  const int4 *items;
  long long nitems;       // this launch drains items [item_begin, nitems)
  long long item_begin;
  unsigned int *queue;     // next item counter (reset per launch)
  const float2 *eo2, *ev2;
  const float *inv_scale;
  double *part;            // [nitems]
  int *err;
};

constexpr int IQ = 4;  // item ring depth between the producer and the consumers
constexpr int TP = TILE + 1;  // padded row of the diagonal-tile transpose buffer (floats)

template <int NSL, int NSTAGE>
__global__ void __launch_bounds__(BATCH_THREADS, 1)
    split_batch_kernel(const __grid_constant__ CUtensorMap tmap, BatchParams P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int STAGE_BYTES = NSL * 2 * PANEL_BYTES;
  constexpr int NEPI = BATCH_EPI;  // epilogue warps: four per TMEM lane quadrant
  uint8_t *stages = base;
  uint64_t *bars = (uint64_t *)(base + NSTAGE * STAGE_BYTES);
  // bars: full[NSTAGE], empty[NSTAGE], t1full, t1empty, t2full, t2empty, drain,
  //       item_full[IQ], item_empty[IQ]
  constexpr int NB = 2 * NSTAGE + 5 + 2 * IQ;
  uint32_t *tmem_slot = (uint32_t *)(bars + NB);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  volatile int *item_q = (volatile int *)(tmem_slot + 2);  // [IQ]
  double *redd = (double *)(((uintptr_t)(tmem_slot + 2 + IQ) + 7) & ~(uintptr_t)7);  // [NEPI]
  // transpose buffer for diagonal tile pairs: 64 rows of T1, padded rows
  float *tbuf = (float *)(base + NSTAGE * STAGE_BYTES + 512);  // [64][TP]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(&bars[0]);
  const uint32_t empty0 = smem_u32(&bars[NSTAGE]);
  const uint32_t t1full = smem_u32(&bars[2 * NSTAGE]);
  const uint32_t t1empty = smem_u32(&bars[2 * NSTAGE + 1]);
  const uint32_t t2full = smem_u32(&bars[2 * NSTAGE + 2]);
  const uint32_t t2empty = smem_u32(&bars[2 * NSTAGE + 3]);
  const uint32_t drain = smem_u32(&bars[2 * NSTAGE + 4]);
  const uint32_t ifull0 = smem_u32(&bars[2 * NSTAGE + 5]);
  const uint32_t iempty0 = smem_u32(&bars[2 * NSTAGE + 5 + IQ]);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(t1full, 1);
    mbar_init(t1empty, NEPI);
    mbar_init(t2full, 1);
    mbar_init(t2empty, NEPI);
    mbar_init(drain, 1);
    for (int s = 0; s < IQ; ++s) {
      mbar_init(ifull0 + 8 * s, 1);
      mbar_init(iempty0 + 8 * s, 1 + NEPI);  // MMA issuer + epilogue warps
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmap) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0) {
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      int armed[NSTAGE];
      for (int s = 0; s < NSTAGE; ++s) armed[s] = -1;
      bool ok = true;
      while (ok) {
        if (!mbar_wait(iempty0 + 8 * islot, iphase ^ 1, abort_flag, P.err, 5)) break;
        const long long id = P.item_begin + (long long)atomicAdd(P.queue, 1u);
        const int qidx = id < P.nitems ? (int)id : -1;
        item_q[islot] = qidx;
        mbar_arrive(ifull0 + 8 * islot);
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        const int4 it = P.items[qidx];
        const FragDesc &F = P.frags[it.x];
        const int i = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
        // T2 = T1 for i == j, and T2 = T1^T (shared-memory transpose) for A == B
        const int ntiles = (i == j || tA == tB) ? 1 : 2;
        for (int t = 0; t < ntiles && ok; ++t) {
          const int colA = (t == 0 ? i : j) * F.nvpad + tA * TILE;
          const int colB = (t == 0 ? j : i) * F.nvpad + tB * TILE;
          for (int kc = 0; kc < F.nks; ++kc) {
            if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err, 1)) {
              ok = false;
              break;
            }
            const uint32_t fb = full0 + 8 * stage;
            mbar_expect_tx(fb, STAGE_BYTES);
            armed[stage] = (int)phase;
            const uint32_t dst = smem_u32(stages + stage * STAGE_BYTES);
            const int rowk = (int)(F.row_base + (long long)kc * F.ncol);
#pragma unroll
            for (int sl = 0; sl < NSL; ++sl) {  // A panels, then the B panels back to back
              tma_load_3d(dst + sl * PANEL_BYTES, &tmap, fb, 0, rowk + colA, sl);
              tma_load_3d(dst + (NSL + sl) * PANEL_BYTES, &tmap, fb, 0, rowk + colB, sl);
            }
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      if (!ok || *abort_flag) {  // drain copies in flight before the CTA can exit
        for (int s = 0; s < NSTAGE; ++s) {
          if (armed[s] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_test(full0 + 8 * s, (uint32_t)armed[s]) && clock64() - t0 < WAIT_BUDGET) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer --------------------------------
    if (lane == 0) {
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      bool ok = true;
      long long nloc = 0;
      while (ok) {
        if (!mbar_wait(ifull0 + 8 * islot, iphase, abort_flag, P.err, 6)) break;
        const int qidx = item_q[islot];
        mbar_arrive(iempty0 + 8 * islot);
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        const int4 it = P.items[qidx];
        const int nks = P.frags[it.x].nks;
        const int i = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
        const int ntiles = (i == j || tA == tB) ? 1 : 2;
        for (int t = 0; t < 2 && ok; ++t) {
          // tile t's accumulators must have been read out for the previous item
          if (nloc > 0 &&
              !mbar_wait(t == 0 ? t1empty : t2empty, (uint32_t)((nloc - 1) & 1), abort_flag, P.err,
                         2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dL0 = tmem + (uint32_t)(t * 2 * TILE);
          const uint32_t dL1 = dL0 + TILE;
          for (int kc = 0; t < ntiles && kc < nks; ++kc) {
            if (!mbar_wait(full0 + 8 * stage, phase, abort_flag, P.err, 3)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sb = smem_u32(stages + stage * STAGE_BYTES);
#pragma unroll
            for (int k16 = 0; k16 < KSTEP / 16; ++k16) {
              const uint32_t koff = k16 * 32;  // bytes inside the 128-byte swizzle row
              const uint64_t a0 = smem_desc(sb + 0 * PANEL_BYTES + koff);
              const uint64_t a1 = smem_desc(sb + 1 * PANEL_BYTES + koff);
              const uint64_t b0 = smem_desc(sb + NSL * PANEL_BYTES + koff);
              const uint64_t b1 = smem_desc(sb + (NSL + 1) * PANEL_BYTES + koff);
              const uint32_t acc = (kc > 0 || k16 > 0) ? 1u : 0u;
              // one N=256 MMA over the stacked B panels [S0b; R1b] fills
              // [L0 | L1]: L0 += S0a S0b (exact integer part), L1 += S0a R1b
              mma_f16_id(dL0, a0, b0, IDESC_N256, acc);
              mma_f16(dL1, a1, b0, 1u);  // R1a S0b
              mma_f16(dL1, a1, b1, 1u);  // R1a R1b
              if (NSL > 2) {
                const uint64_t a2 = smem_desc(sb + 2 * PANEL_BYTES + koff);
                const uint64_t b2 = smem_desc(sb + (NSL + 2) * PANEL_BYTES + koff);
                mma_f16(dL1, a0, b2, 1u);  // S0a R2b
                mma_f16(dL1, a2, b0, 1u);  // R2a S0b
              }
            }
            mma_commit(empty0 + 8 * stage);  // frees the stage when these MMAs finish
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          mma_commit(t == 0 ? t1full : t2full);  // tile t of this item is complete
        }
        if (!ok) break;
        ++nloc;
      }
      // drain: all MMAs issued by this thread complete before TMEM is freed
      mma_commit(drain);
      const long long t0 = clock64();
      while (!mbar_test(drain, 0) && clock64() - t0 < WAIT_BUDGET) {
      }
    }
  } else {
    // ------------------------------ epilogue ----------------------------------
    const int ew = warp - 2;             // 0..15
    const int quad = warp & 3;           // TMEM lane quadrant this warp may access
    const int cbase = (ew >> 2) * 32;    // the 32 columns of the tile this warp reads
    const int row = quad * 32 + lane;    // tile row = a offset
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int islot = 0;
    uint32_t iphase = 0;
    long long nloc = 0;
    while (true) {
      const bool w0 = mbar_wait(ifull0 + 8 * islot, iphase, abort_flag, P.err, 7);
      if (epi_any512(!w0)) break;
      const int qidx = item_q[islot];
      __syncwarp();
      if (lane == 0) mbar_arrive(iempty0 + 8 * islot);
      if (++islot == IQ) {
        islot = 0;
        iphase ^= 1;
      }
      if (qidx < 0) break;
      const int4 it = P.items[qidx];
      const FragDesc &F = P.frags[it.x];
      const int i = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
      const bool same = (i == j), diag = (tA == tB);
      const int nvpad = F.nvpad;
      const int a = tA * TILE + row;
      const float *scl = P.inv_scale + F.col_base;
      const float sa1 = scl[i * nvpad + a];  // scale of column (a,i)
      const float sa2 = scl[j * nvpad + a];  // scale of column (a,j)
      const float *sbj = scl + j * nvpad + tB * TILE + cbase;
      const float *sbi = scl + i * nvpad + tB * TILE + cbase;
      const float2 *evb = P.ev2 + F.ev_off + tB * TILE + cbase;
      // ---- T1 -> registers, then hand its TMEM back to the MMA issuer ----
      const bool w1 = mbar_wait(t1full, (uint32_t)(nloc & 1), abort_flag, P.err, 4);
      if (epi_any512(!w1)) break;
      tc_fence_after();
      const uint32_t t1 = tmem + lane_off + cbase;
      float g1[32];
#pragma unroll
      for (int c0 = 0; c0 < 32; c0 += 16) {
        float l0[16], l1[16];
        tmem_ld16(t1 + c0, l0);
        tmem_ld16(t1 + TILE + c0, l1);
        tmem_wait_ld();
#pragma unroll
        for (int k = 0; k < 16; ++k) g1[c0 + k] = (l0[k] + l1[k]) * (sa1 * sbj[c0 + k]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(t1empty);
      // ---- denominators ----
      const float2 ea = P.ev2[F.ev_off + a];
      const float2 ei = P.eo2[F.eo_off + i], ej = P.eo2[F.eo_off + j];
      // e_i + e_j in hi/lo form (two-sum of the hi parts, lo parts added)
      const float sh = ei.x + ej.x;
      const float bv = sh - ei.x;
      const float sl = (ei.x - (sh - bv)) + (ej.x - bv) + ei.y + ej.y;
      // per-row part of the denominator, again as an exact two-sum
      const float dh0 = sh - ea.x;
      const float bw = dh0 - sh;
      const float dl0 = ((sh - (dh0 - bw)) + (-ea.x - bw)) + (sl - ea.y);
      // ---- T2 and the energy terms ----
      const bool w2 = mbar_wait(t2full, (uint32_t)(nloc & 1), abort_flag, P.err, 8);
      if (epi_any512(!w2)) break;
      tc_fence_after();
      // items that do not read T2 (i = j, or A = B with T2 = T1^T) hand it
      // back to the MMA issuer at once
      bool t2_held = true;
      if (same || diag) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(t2empty);
        t2_held = false;
      }
      const uint32_t t2 = tmem + lane_off + 2 * TILE + cbase;
      // one 16-column chunk of energy terms, g2 supplied by `g2at(k)`
      auto terms = [&](int c0, const float *g2) -> float {
        float ef = 0.0f;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const float2 eb = evb[c0 + k];
          const float x1 = g1[c0 + k], x2 = g2[k];
          // d = (dh0 + dl0) - (eb.x + eb.y) with the leading subtraction exact
          const float dh = dh0 - eb.x;
          const float bz = dh - dh0;
          const float d = dh + (((dh0 - (dh - bz)) + (-eb.x - bz)) + (dl0 - eb.y));
          const float r = rcp_denom(d);
          const float num = diag ? x1 * fmaf(2.0f, x1, -x2) : 2.0f * fmaf(x1, x1 - x2, x2 * x2);
          ef = fmaf(num, r, ef);
        }
        return ef;
      };
      double eacc = 0.0;
      if (diag && !same) {
        // T2[a,b] = g_ij(b,a) = T1[b,a]: transpose T1 through shared memory in
        // two 64-row passes; pass h serves the warps that own columns [64h,64h+64)
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
          asm volatile("bar.sync 1, 512;" ::: "memory");
          if ((row >> 6) == h) {
            float *dst = tbuf + (row - 64 * h) * TP + cbase;
#pragma unroll
            for (int k = 0; k < 32; ++k) dst[k] = g1[k];
          }
          asm volatile("bar.sync 1, 512;" ::: "memory");
          if ((cbase >> 6) == h) {
#pragma unroll
            for (int c0 = 0; c0 < 32; c0 += 16) {
              float g2[16];
#pragma unroll
              for (int k = 0; k < 16; ++k) g2[k] = tbuf[(cbase - 64 * h + c0 + k) * TP + row];
              eacc += (double)terms(c0, g2);
            }
          }
        }
      } else {
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
          float g2[16];
          if (same) {
#pragma unroll
            for (int k = 0; k < 16; ++k) g2[k] = g1[c0 + k];
          } else {
            float l0[16], l1[16];
            tmem_ld16(t2 + c0, l0);
            tmem_ld16(t2 + TILE + c0, l1);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 16; ++k) g2[k] = (l0[k] + l1[k]) * (sa2 * sbi[c0 + k]);
          }
          eacc += (double)terms(c0, g2);
        }
      }
      if (t2_held) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(t2empty);
      }
      // reduce the item's energy over the epilogue threads
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
      if (lane == 0) redd[ew] = eacc;
      asm volatile("bar.sync 1, 512;" ::: "memory");
      if (ew == 0 && lane == 0) {
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < NEPI; ++w) tot += redd[w];
        P.part[it.w] = tot;
      }
      asm volatile("bar.sync 1, 512;" ::: "memory");
      ++nloc;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// ==========================================================================
// Paired-CTA form of the energy kernel (cta_group::2 on a cluster of two
// CTAs, M = 256).  The two CTAs of a pair evaluate the occupied pairs
// (i0, j) and (i0 + 1, j) for the same tile pair (A, B):
//   T1  = G_ij[A,B] = C_iA^T C_jB   (a on the TMEM lanes, b on the columns)
//   T2' = G_ij[B,A] = C_iB^T C_jA   (b on the lanes, a on the columns)
// Both products of an item have the same B operand in the two CTAs (C_jB,
// then C_jA), which the pair splits between its shared memories.  This
// kernel uses a third slice plane V = fp16(C*s) and folds the two R1a terms
// into one product, R1a S0b + R1a R1b = R1a V - R1a (V - S0 - R1), so a K16
// step is two MMAs (three products instead of four):
//   256x256: S0a x [S0b; R1b] -> [L0 | L1]   (B rows 0..127 = S0b from rank 0,
//                                             rows 128..255 = R1b from rank 1)
//   256x128: R1a x Vb -> L1                   (64 rows of V from each rank)
// The dropped term sum_k R1a (Vb - S0b - R1b) is a product of two
// independent rounding residues for distinct columns (a,i) != (b,j), an
// unbiased error of ~2^-21 of g that averages out of the pair energies; for
// the same column it is a sum of R1 times its own rounding error, a bias,
// which the slicing kernel computes per column (dcorr) and the epilogue
// subtracts from g_ii(a,a).  Each SM's tensor core reads 14 KB of operands
// per step (the one-CTA kernel: 28 KB for four products).
// T2' is transposed through shared memory in the epilogue, so that g_ij(a,b)
// and g_ij(b,a) meet in one thread.
// A pair item with i0 + 1 > j runs its second CTA as a dummy (results
// discarded); i0 == j (then the second CTA is a dummy) and A == B need only
// T1.  The even CTA of the pair (rank 0) owns the work queue, the TMA full
// barriers (both CTAs' copies complete on them), the MMA issue and the
// accumulator-empty barriers; its commits are multicast to both CTAs.  Every
// wait is bounded; a timeout in either CTA aborts both.
// --------------------------------------------------------------------------
constexpr int BHALF = TILE / 2;                  // B rows of an N=128 operand per CTA
constexpr int BPANEL_BYTES = BHALF * KSTEP * 2;  // 8 KB
// per-CTA stage: A panels S0a, R1a (16 KB each); Y = 128 rows of the N=256
// operand (rank 0: S0b, rank 1: R1b); W = 64 rows of Vb
constexpr int PAIR_STAGE_BYTES = 3 * PANEL_BYTES + BPANEL_BYTES;  // 56 KB
// kind::f16, A = B = F16, D = F32, K-major, M = 256 (pair), N = 128 / 256
constexpr uint32_t IDESC_PAIR = (1u << 4) | ((uint32_t)(TILE >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
constexpr uint32_t IDESC_PAIR_N256 = (1u << 4) | ((uint32_t)(256 >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// shared::cluster address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_shared(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}

__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr)
               : "memory");
}

__device__ __forceinline__ bool mbar_test_cl(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void st_remote_u32(uint32_t cluster_addr, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr), "r"(v) : "memory");
}

// TMA load into this CTA's shared memory whose completion is counted on the
// pair's (rank 0) barrier
__device__ __forceinline__ void tma_load_3d_pair(uint32_t dst, const CUtensorMap *map,
                                                 uint32_t bar_cluster, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
      "l"((uint64_t)map), "r"(bar_cluster), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

__device__ __forceinline__ void mma_f16_pair(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                             uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

// arrive on the barrier at this shared offset in both CTAs of the pair once
// all previously issued MMAs of this thread have completed
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(bar),
      "h"((uint16_t)3)
      : "memory");
}

// Bounded wait that also aborts the peer CTA on a timeout.
__device__ __forceinline__ bool pair_wait(uint32_t bar, uint32_t parity, bool cluster_scope,
                                          volatile int *abort_flag, uint32_t abort_peer, int *err,
                                          int code) {
  const long long t0 = clock64();
  while (!(cluster_scope ? mbar_test_cl(bar, parity) : mbar_test(bar, parity))) {
    if (*abort_flag) return false;
    if (clock64() - t0 > WAIT_BUDGET) {
      *abort_flag = 1;
      st_remote_u32(abort_peer, 1u);
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

struct PairParams {
  const FragDesc *frags;
  const int4 *items;     // {fragment, i0 | j << 16, tA | tB << 16, tile pair index}
  long long nitems;      // this launch drains items [item_begin, nitems)
  long long item_begin;
  const float *dcorr;    // per column: sum over K of R1 (V - S0 - R1)
  unsigned int *queue;   // next item counter (reset per launch)
  const float2 *eo2, *ev2;
  const float *inv_scale;
  double *part;          // indexed like split_batch_kernel's work items
  float *xbuf;           // GX form: one 128x128 FP32 exchange tile per CTA of the grid
  int *err;
};

// Shared memory of split_pair_kernel<NSTAGE, GX>: the stage ring, barriers and
// item ring, and (GX = false) the 64-row transpose buffer.  With the exchange
// tile transposed through global scratch (GX = true) a fourth 56 KB stage
// fits in the 227 KB a CTA may hold.
constexpr int pair_smem_bytes(int nstage, bool gx) {
  return nstage * PAIR_STAGE_BYTES + 1024 + 512 + (gx ? 0 : 64 * TP * 4);
}

// Exchange-tile transpose through memory, for the GX form: each thread stores
// its 64 values of tile row `row` (columns [cbase, cbase+64)) as 16-byte
// vectors, and after a barrier reads column `row` back 16 values at a time,
// coalesced across the warp.  The .cg forms keep the round trip in L2, so no
// SM-local cache line of the previous item's tile is ever read.
__device__ __forceinline__ void st_cg4(float *p, float a, float b, float c, float d) {
  asm volatile("st.global.cg.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}
__device__ __forceinline__ float ld_cg(const float *p) {
  float v;
  asm volatile("ld.global.cg.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}

template <int NSTAGE, bool GX>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NTHREADS, 1)
    split_pair_kernel(const __grid_constant__ CUtensorMap tmA,
                      const __grid_constant__ CUtensorMap tmB, PairParams P) {
  constexpr int STAGE_BYTES = PAIR_STAGE_BYTES;
  constexpr int NEPI = 8;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *stages = base;
  uint64_t *bars = (uint64_t *)(base + NSTAGE * STAGE_BYTES);
  // bars: full[NSTAGE], empty[NSTAGE], t1full, t1empty, t2full, t2empty, drain,
  //       item_full[IQ], item_empty[IQ]
  constexpr int NB = 2 * NSTAGE + 5 + 2 * IQ;
  uint32_t *tmem_slot = (uint32_t *)(bars + NB);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  volatile int *item_q = (volatile int *)(tmem_slot + 2);  // [IQ]
  double *redd = (double *)(((uintptr_t)(tmem_slot + 2 + IQ) + 7) & ~(uintptr_t)7);  // [NEPI]
  float *tbuf = (float *)(base + NSTAGE * STAGE_BYTES + 512);  // [64][TP]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const bool leader = rank == 0;
  const uint32_t full0 = smem_u32(&bars[0]);
  const uint32_t empty0 = smem_u32(&bars[NSTAGE]);
  const uint32_t t1full = smem_u32(&bars[2 * NSTAGE]);
  const uint32_t t1empty = smem_u32(&bars[2 * NSTAGE + 1]);
  const uint32_t t2full = smem_u32(&bars[2 * NSTAGE + 2]);
  const uint32_t t2empty = smem_u32(&bars[2 * NSTAGE + 3]);
  const uint32_t drain = smem_u32(&bars[2 * NSTAGE + 4]);
  const uint32_t ifull0 = smem_u32(&bars[2 * NSTAGE + 5]);
  const uint32_t iempty0 = smem_u32(&bars[2 * NSTAGE + 5 + IQ]);
  // the pair's shared barriers live in rank 0
  const uint32_t full0_L = map_shared(full0, 0);
  const uint32_t t1empty_L = map_shared(t1empty, 0);
  const uint32_t t2empty_L = map_shared(t2empty, 0);
  const uint32_t iempty0_L = map_shared(iempty0, 0);
  const uint32_t abort_peer = map_shared(smem_u32((const void *)abort_flag), rank ^ 1u);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full0 + 8 * s, 1);   // rank 0: its producer's arrive + both CTAs' bytes
      mbar_init(empty0 + 8 * s, 1);  // multicast MMA commit
    }
    mbar_init(t1full, 1);
    mbar_init(t1empty, 2 * NEPI);  // epilogue warps of both CTAs
    mbar_init(t2full, 1);
    mbar_init(t2empty, 2 * NEPI);
    mbar_init(drain, 1);
    for (int s = 0; s < IQ; ++s) {
      mbar_init(ifull0 + 8 * s, 1);
      mbar_init(iempty0 + 8 * s, 2 + 2 * NEPI);  // MMA issuer, peer producer, all epilogue warps
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // both CTAs' barriers are initialised before any remote access
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // --------------------- TMA producers (both CTAs) ---------------------
    if (lane == 0) {
      const uint32_t item_q_peer = map_shared(smem_u32((const void *)item_q), 1);
      const uint32_t ifull0_peer = map_shared(ifull0, 1);
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      uint32_t armed = 0, armed_par = 0;  // rank 0: stages with copies expected, and parity
      bool ok = true;
      while (ok) {
        int qidx;
        if (leader) {
          if (!pair_wait(iempty0 + 8 * islot, iphase ^ 1, true, abort_flag, abort_peer, P.err, 5))
            break;
          const long long id = P.item_begin + (long long)atomicAdd(P.queue, 1u);
          qidx = id < P.nitems ? (int)id : -1;
          item_q[islot] = qidx;
          st_remote_u32(item_q_peer + 4 * islot, (uint32_t)qidx);
          mbar_arrive(ifull0 + 8 * islot);
          mbar_arrive_remote(ifull0_peer + 8 * islot);
        } else {
          if (!pair_wait(ifull0 + 8 * islot, iphase, true, abort_flag, abort_peer, P.err, 5))
            break;
          qidx = item_q[islot];
          mbar_arrive_remote(iempty0_L + 8 * islot);
        }
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        const int4 it = P.items[qidx];
        const FragDesc &F = P.frags[it.x];
        const int i0 = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
        const int i = (i0 + (int)rank <= j) ? i0 + (int)rank : i0;  // a dummy loads i0's panels
        const int ntiles = (tA == tB || i0 == j) ? 1 : 2;
        for (int t = 0; t < ntiles && ok; ++t) {
          const int colA = i * F.nvpad + (t == 0 ? tA : tB) * TILE;
          const int colB = j * F.nvpad + (t == 0 ? tB : tA) * TILE;
          const int colH = colB + BHALF * (int)rank;  // this rank's half of the B rows
          for (int kc = 0; kc < F.nks; ++kc) {
            if (!pair_wait(empty0 + 8 * stage, phase ^ 1, false, abort_flag, abort_peer, P.err, 1)) {
              ok = false;
              break;
            }
            if (leader) {
              mbar_expect_tx(full0 + 8 * stage, 2 * STAGE_BYTES);
              armed |= 1u << stage;
              armed_par = (armed_par & ~(1u << stage)) | (phase << stage);
            }
            const uint32_t dst = smem_u32(stages + stage * STAGE_BYTES);
            const uint32_t fb = full0_L + 8 * stage;
            const int rowk = (int)(F.row_base + (long long)kc * F.ncol);
            tma_load_3d_pair(dst, &tmA, fb, 0, rowk + colA, 0);                // S0a
            tma_load_3d_pair(dst + PANEL_BYTES, &tmA, fb, 0, rowk + colA, 1);  // R1a
            tma_load_3d_pair(dst + 2 * PANEL_BYTES, &tmA, fb, 0, rowk + colB, (int)rank);  // Y
            tma_load_3d_pair(dst + 3 * PANEL_BYTES, &tmB, fb, 0, rowk + colH, 2);  // W: V half
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      if (leader && (!ok || *abort_flag)) {  // copies in flight complete before the pair exits
        for (int s = 0; s < NSTAGE; ++s) {
          if (!((armed >> s) & 1u)) continue;
          const long long t0 = clock64();
          while (!mbar_test(full0 + 8 * s, (armed_par >> s) & 1u) && clock64() - t0 < WAIT_BUDGET) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // --------------------- MMA issuer (rank 0 only) ----------------------
    if (lane == 0 && leader) {
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      bool ok = true;
      long long nloc = 0;
      while (ok) {
        if (!pair_wait(ifull0 + 8 * islot, iphase, false, abort_flag, abort_peer, P.err, 6)) break;
        const int qidx = item_q[islot];
        mbar_arrive_remote(iempty0_L + 8 * islot);
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        const int4 it = P.items[qidx];
        const int nks = P.frags[it.x].nks;
        const int i0 = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
        const int ntiles = (tA == tB || i0 == j) ? 1 : 2;
        for (int t = 0; t < 2 && ok; ++t) {
          // both CTAs' epilogues have read tile t of the previous item
          if (nloc > 0 && !pair_wait(t == 0 ? t1empty : t2empty, (uint32_t)((nloc - 1) & 1), true,
                                     abort_flag, abort_peer, P.err, 2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dL0 = tmem + (uint32_t)(t * 2 * TILE);
          const uint32_t dL1 = dL0 + TILE;
          for (int kc = 0; t < ntiles && kc < nks; ++kc) {
            if (!pair_wait(full0 + 8 * stage, phase, false, abort_flag, abort_peer, P.err, 3)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sb = smem_u32(stages + stage * STAGE_BYTES);
#pragma unroll
            for (int k16 = 0; k16 < KSTEP / 16; ++k16) {
              const uint32_t koff = k16 * 32;  // bytes inside the 128-byte swizzle row
              const uint64_t a0 = smem_desc(sb + koff);
              const uint64_t a1 = smem_desc(sb + PANEL_BYTES + koff);
              const uint64_t by = smem_desc(sb + 2 * PANEL_BYTES + koff);
              const uint64_t bw = smem_desc(sb + 3 * PANEL_BYTES + koff);
              const uint32_t acc = (kc > 0 || k16 > 0) ? 1u : 0u;
              // [L0 | L1] += S0a x [S0b; R1b]: exact integer part and S0a R1b
              mma_f16_pair(dL0, a0, by, IDESC_PAIR_N256, acc);
              mma_f16_pair(dL1, a1, bw, IDESC_PAIR, 1u);  // R1a V (= R1a S0b + R1a R1b + R1a eps)
            }
            mma_commit_pair(empty0 + 8 * stage);  // frees the stage in both CTAs
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          mma_commit_pair(t == 0 ? t1full : t2full);
        }
        if (!ok) break;
        ++nloc;
      }
      mma_commit_pair(drain);  // both CTAs learn when the last MMA has completed
    }
  } else {
    // --------------------- epilogue (both CTAs) ---------------------------
    const int ew = warp - 2;           // 0..7
    const int quad = warp & 3;         // TMEM lane quadrant this warp may access
    const int cbase = (ew >> 2) * 64;  // column half of the tile this warp reads
    const int row = quad * 32 + lane;  // TMEM lane = tile row
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    int islot = 0;
    uint32_t iphase = 0;
    long long nloc = 0;
    while (true) {
      const bool w0 = pair_wait(ifull0 + 8 * islot, iphase, true, abort_flag, abort_peer, P.err, 7);
      if (epi_any(!w0)) break;
      const int qidx = item_q[islot];
      __syncwarp();
      if (lane == 0) mbar_arrive_remote(iempty0_L + 8 * islot);
      if (++islot == IQ) {
        islot = 0;
        iphase ^= 1;
      }
      if (qidx < 0) break;
      const int4 it = P.items[qidx];
      const FragDesc &F = P.frags[it.x];
      const int i0 = it.y & 0xFFFF, j = it.y >> 16, tA = it.z & 0xFFFF, tB = it.z >> 16;
      const bool dummy = i0 + (int)rank > j;
      const int i = dummy ? i0 : i0 + (int)rank;
      const bool same = (i == j), diag = (tA == tB);
      const int nvpad = F.nvpad;
      const int a = tA * TILE + row;
      const float *scl = P.inv_scale + F.col_base;
      const float sa1 = scl[i * nvpad + a];                    // column (a,i)
      const float *sbj = scl + j * nvpad + tB * TILE + cbase;  // columns (b,j)
      const float2 *evb = P.ev2 + F.ev_off + tB * TILE + cbase;
      // ---- T1 -> registers, then release it ----
      const bool w1 = pair_wait(t1full, (uint32_t)(nloc & 1), false, abort_flag, abort_peer, P.err, 4);
      if (epi_any(!w1)) break;
      tc_fence_after();
      const uint32_t t1 = tmem + lane_off + cbase;
      float g1[64];
#pragma unroll
      for (int c0 = 0; c0 < 64; c0 += 16) {
        float l0[16], l1[16];
        tmem_ld16(t1 + c0, l0);
        tmem_ld16(t1 + TILE + c0, l1);
        tmem_wait_ld();
#pragma unroll
        for (int k = 0; k < 16; ++k) g1[c0 + k] = (l0[k] + l1[k]) * (sa1 * sbj[c0 + k]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive_remote(t1empty_L);
      if (same && diag && !dummy) {
        // g_ii(a,a): remove the same-column bias of the folded R1 V product
        const float corr = P.dcorr[F.col_base + i * nvpad + a] * (sa1 * sa1);
        const int kd = row - cbase;  // this row's diagonal element in the warp's column half
#pragma unroll
        for (int k = 0; k < 64; ++k)
          if (k == kd) g1[k] -= corr;
      }
      // ---- denominators (as split_batch_kernel) ----
      const float2 ea = P.ev2[F.ev_off + a];
      const float2 ei = P.eo2[F.eo_off + i], ej = P.eo2[F.eo_off + j];
      const float sh = ei.x + ej.x;
      const float bv = sh - ei.x;
      const float sl = (ei.x - (sh - bv)) + (ej.x - bv) + ei.y + ej.y;
      const float dh0 = sh - ea.x;
      const float bw = dh0 - sh;
      const float dl0 = ((sh - (dh0 - bw)) + (-ea.x - bw)) + (sl - ea.y);
      auto terms = [&](int c0, const float *g2) -> float {
        float ef = 0.0f;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const float2 eb = evb[c0 + k];
          const float x1 = g1[c0 + k], x2 = g2[k];
          const float dh = dh0 - eb.x;
          const float bz = dh - dh0;
          const float d = dh + (((dh0 - (dh - bz)) + (-eb.x - bz)) + (dl0 - eb.y));
          const float r = rcp_denom(d);
          const float num = diag ? x1 * fmaf(2.0f, x1, -x2) : 2.0f * fmaf(x1, x1 - x2, x2 * x2);
          ef = fmaf(num, r, ef);
        }
        return ef;
      };
      // ---- T2' and the energy terms ----
      const bool w2 = pair_wait(t2full, (uint32_t)(nloc & 1), false, abort_flag, abort_peer, P.err, 8);
      if (epi_any(!w2)) break;
      tc_fence_after();
      // each warp hands T2' back to the MMA issuer as soon as it has read its
      // rows (or at once when this item does not read T2'), so that the next
      // item's second chain can start while the energy terms are formed
      bool t2_held = true;
      auto release_t2 = [&]() {
        if (t2_held) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_remote(t2empty_L);
          t2_held = false;
        }
      };
      if (dummy || same || diag) release_t2();
      double eacc = 0.0;
      if (!dummy) {
        if (same) {  // g_ii is symmetric
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 16) {
            float g2[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) g2[k] = g1[c0 + k];
            eacc += (double)terms(c0, g2);
          }
        } else {
          // g2(a,b) = g_ij(b,a): T1 transposed (A == B) or T2' = G_ij[B,A]
          // transposed, through shared memory in two 64-row passes; pass h
          // serves the warps that own columns [64h, 64h+64)
          const uint32_t t2 = tmem + lane_off + 2 * TILE + cbase;
          const float sbi = scl[i * nvpad + tB * TILE + row];      // T2' row (b,i)
          const float *saj = scl + j * nvpad + tA * TILE + cbase;  // T2' columns (a,j)
          if constexpr (GX) {
            // every thread stores row `row` of the tile to transpose (T1 when
            // A == B, else T2'), then reads column `row` of it
            float *X = P.xbuf + (size_t)blockIdx.x * (TILE * TILE);
            float *dst = X + row * TILE + cbase;
            if (diag) {
#pragma unroll
              for (int k = 0; k < 64; k += 4) st_cg4(dst + k, g1[k], g1[k + 1], g1[k + 2], g1[k + 3]);
            } else {
#pragma unroll
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float l0[16], l1[16];
                tmem_ld16(t2 + c0, l0);
                tmem_ld16(t2 + TILE + c0, l1);
                tmem_wait_ld();
                float v[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) v[k] = (l0[k] + l1[k]) * (sbi * saj[c0 + k]);
#pragma unroll
                for (int k = 0; k < 16; k += 4) st_cg4(dst + c0 + k, v[k], v[k + 1], v[k + 2], v[k + 3]);
              }
              release_t2();
            }
            asm volatile("bar.sync 1, 256;" ::: "memory");
            const float *src = X + (size_t)cbase * TILE + row;
            float ga[16], gb[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) ga[k] = ld_cg(src + k * TILE);
#pragma unroll
            for (int c0 = 0; c0 < 64; c0 += 32) {
#pragma unroll
              for (int k = 0; k < 16; ++k) gb[k] = ld_cg(src + (c0 + 16 + k) * TILE);
              eacc += (double)terms(c0, ga);
              if (c0 + 32 < 64) {
#pragma unroll
                for (int k = 0; k < 16; ++k) ga[k] = ld_cg(src + (c0 + 32 + k) * TILE);
              }
              eacc += (double)terms(c0 + 16, gb);
            }
          } else {
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            asm volatile("bar.sync 1, 256;" ::: "memory");
            if ((row >> 6) == h) {
              float *dst = tbuf + (row - 64 * h) * TP + cbase;
              if (diag) {
#pragma unroll
                for (int k = 0; k < 64; ++k) dst[k] = g1[k];
              } else {
#pragma unroll
                for (int c0 = 0; c0 < 64; c0 += 16) {
                  float l0[16], l1[16];
                  tmem_ld16(t2 + c0, l0);
                  tmem_ld16(t2 + TILE + c0, l1);
                  tmem_wait_ld();
#pragma unroll
                  for (int k = 0; k < 16; ++k) dst[c0 + k] = (l0[k] + l1[k]) * (sbi * saj[c0 + k]);
                }
                release_t2();
              }
            }
            asm volatile("bar.sync 1, 256;" ::: "memory");
            if ((cbase >> 6) == h) {
#pragma unroll
              for (int c0 = 0; c0 < 64; c0 += 16) {
                float g2[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) g2[k] = tbuf[(c0 + k) * TP + row];
                eacc += (double)terms(c0, g2);
              }
            }
          }
          }
        }
      }
      release_t2();
      // reduce the item's energy over the epilogue threads
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
      if (lane == 0) redd[ew] = eacc;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (ew == 0 && lane == 0 && !dummy) {
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < NEPI; ++w) tot += redd[w];
        const long long p = (long long)j * (j + 1) / 2 + i;
        P.part[F.item_base + p * F.ntp + it.w] = tot;
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
      ++nloc;
    }
  }
  __syncthreads();
  if (warp == 1 && lane == 0) {
    // the last MMA of the pair has completed (it may write this CTA's TMEM)
    const long long t0 = clock64();
    while (!mbar_test(drain, 0) && clock64() - t0 < WAIT_BUDGET) {
    }
  }
  if (*abort_flag) {
    // after an abort the peer may still have copies in flight into its own
    // shared memory (their completion is counted in rank 0): give them time
    // to land before either CTA exits
    const long long t0 = clock64();
    while (clock64() - t0 < 4000000LL) {
    }
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// Pair items of a group: per fragment, for each j the i0 = 0, 2, 4, ... <= j,
// times the tile pairs.  C(j) = number of pair items (without the tile-pair
// factor) before column j = floor(j/2) * floor(j/2 + 1) for even j and
// (floor(j/2) + 1)^2 for odd j.
__host__ __device__ inline long long pair_items_before(long long j) {
  const long long m = j / 2;
  return (j % 2 == 0) ? m * (m + 1) : (m + 1) * (m + 1);
}

__global__ void build_pair_items_kernel(const FragDesc *__restrict__ fr, int nfrag,
                                        long long nitems, int4 *__restrict__ items) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nitems) return;
  int lo = 0, hi = nfrag - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (fr[mid].pitem_base <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const FragDesc &F = fr[lo];
  const long long loc = t - F.pitem_base;
  const long long p2 = loc / F.ntp;
  const int q = (int)(loc % F.ntp);
  int j = (int)(2.0 * sqrt((double)p2));
  if (j > F.nocc - 1) j = F.nocc - 1;
  while (j > 0 && pair_items_before(j) > p2) --j;
  while (j + 1 < F.nocc && pair_items_before(j + 1) <= p2) ++j;
  const int i0 = (int)(2 * (p2 - pair_items_before(j)));
  int tA, tB;
  decode_tri(q, tA, tB);
  items[t] = make_int4(lo, i0 | (j << 16), tA | (tB << 16), q);
}

// ==========================================================================
// Local-orbital fragment energy on the tensor cores (split form):
//   sum_ij,ab g_ij^ab / D (2 gt_ij^ab - gt_ij^ba),
// g from Calpha C, gt from its projected copy Ct (both sliced like Calpha).
// Work item = (pair i<=j, tile pair A<=B, column half h): rows a in block A
// (128), columns b in the h-th 64-column half of block B.  Four 128x64 tiles
// per item: T1 = C_iA^T C_jB, T2 = C_jA^T C_iB, U1 = Ct_iA^T Ct_jB,
// U2 = Ct_jA^T Ct_iB, each with L0/L1 accumulators: 8 x 64 = 512 TMEM columns.
// Diagonal tile pairs compute T2/U2 too (no transpose), so each ordered (a,b)
// of A x A is met once over the two halves; i = j reuses T1/U1.
// Roles as in split_batch_kernel; the MMA issuer waits for the epilogue to
// free all four tiles before the next item (no accumulator double-buffer).
// --------------------------------------------------------------------------
constexpr int HALF = 64;
constexpr int HPANEL_BYTES = HALF * KSTEP * 2;  // 8 KB

struct EosParams {
  const float *inv;          // inverse scales: C columns [0, ncol), Ct columns [ncol, 2 ncol)
  const float2 *eo2, *ev2;   // hi/lo orbital energies (ev2 padded to nvpad)
  long long nitems;
  unsigned int *queue;
  double *part;              // [nitems]
  int *err;
  int nocc, nvirt, nvpad, nks, ntp, ncol;
  int rowC, rowCt;           // first slice row of C and of Ct (per plane)
  const float *dcorr;        // one residual slice: per column sum_k R1 (V - S0 - R1)
};

// One residual slice adds the V plane (three products per element pair, as
// in split_pair_kernel): a stage holds S0a, R1a (128 rows) and S0b, R1b, Vb
// (64 rows).
constexpr int eos_stage_bytes(int nsl) {
  return nsl * PANEL_BYTES + (nsl + (nsl == 2 ? 1 : 0)) * HPANEL_BYTES;
}

__device__ __forceinline__ void eos_decode(const EosParams &P, long long id, int &i, int &j,
                                           int &tA, int &tB, int &h) {
  const int per = 2 * P.ntp;
  const int p = (int)(id / per), r = (int)(id % per);
  decode_pair(p, i, j);
  decode_tri(r >> 1, tA, tB);
  h = r & 1;
}

template <int NSL, int NSTAGE>
__global__ void __launch_bounds__(NTHREADS, 1)
    split_eos_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     EosParams P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr bool VP = (NSL == 2);  // V plane: R1a S0b + R1a R1b folded into R1a V
  constexpr int STAGE_BYTES = eos_stage_bytes(NSL);
  constexpr int NEPI = 8;
  uint8_t *stages = base;
  uint64_t *bars = (uint64_t *)(base + NSTAGE * STAGE_BYTES);
  // bars: full[NSTAGE], empty[NSTAGE], tfull[4], tempty[4], drain, item_full[IQ],
  //       item_empty[IQ]
  constexpr int NB = 2 * NSTAGE + 9 + 2 * IQ;
  uint32_t *tmem_slot = (uint32_t *)(bars + NB);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  volatile long long *item_q =
      (volatile long long *)(((uintptr_t)(tmem_slot + 2) + 7) & ~(uintptr_t)7);  // [IQ]
  double *redd = (double *)(item_q + IQ);                                       // [NEPI]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(&bars[0]);
  const uint32_t empty0 = smem_u32(&bars[NSTAGE]);
  const uint32_t tfull0 = smem_u32(&bars[2 * NSTAGE]);       // + 8 t
  const uint32_t tempty0 = smem_u32(&bars[2 * NSTAGE + 4]);  // + 8 t
  const uint32_t drain = smem_u32(&bars[2 * NSTAGE + 8]);
  const uint32_t ifull0 = smem_u32(&bars[2 * NSTAGE + 9]);
  const uint32_t iempty0 = smem_u32(&bars[2 * NSTAGE + 9 + IQ]);

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int t = 0; t < 4; ++t) {
      mbar_init(tfull0 + 8 * t, 1);
      mbar_init(tempty0 + 8 * t, NEPI);
    }
    mbar_init(drain, 1);
    for (int s = 0; s < IQ; ++s) {
      mbar_init(ifull0 + 8 * s, 1);
      mbar_init(iempty0 + 8 * s, 1 + NEPI);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // tiles in issue order o = 0..3: T1 (C), U1 (Ct), T2 (C), U2 (Ct), i.e. tile
  // t = 2 (o & 1) + (o >> 1); i = j items skip T2/U2

  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0) {
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      int armed[NSTAGE];
      for (int s = 0; s < NSTAGE; ++s) armed[s] = -1;
      bool ok = true;
      while (ok) {
        if (!mbar_wait(iempty0 + 8 * islot, iphase ^ 1, abort_flag, P.err, 5)) break;
        const long long id = (long long)atomicAdd(P.queue, 1u);
        const long long qidx = id < P.nitems ? id : -1;
        item_q[islot] = qidx;
        mbar_arrive(ifull0 + 8 * islot);
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        int i, j, tA, tB, h;
        eos_decode(P, qidx, i, j, tA, tB, h);
        const bool same = (i == j);
        for (int o = 0; o < 4 && ok; ++o) {
          const int t = ((o & 1) << 1) | (o >> 1);
          if (same && (t & 1)) continue;  // T2 = T1, U2 = U1
          const int rowbase = (t < 2) ? P.rowC : P.rowCt;
          const int ia = (t & 1) ? j : i, ib = (t & 1) ? i : j;
          const int colA = ia * P.nvpad + tA * TILE;
          const int colB = ib * P.nvpad + tB * TILE + h * HALF;
          for (int kc = 0; kc < P.nks; ++kc) {
            if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err, 1)) {
              ok = false;
              break;
            }
            const uint32_t fb = full0 + 8 * stage;
            mbar_expect_tx(fb, STAGE_BYTES);
            armed[stage] = (int)phase;
            const uint32_t dst = smem_u32(stages + stage * STAGE_BYTES);
            const int rowk = rowbase + kc * P.ncol;
#pragma unroll
            for (int sl = 0; sl < NSL; ++sl) {
              tma_load_3d(dst + sl * PANEL_BYTES, &tmA, fb, 0, rowk + colA, sl);
              tma_load_3d(dst + NSL * PANEL_BYTES + sl * HPANEL_BYTES, &tmB, fb, 0, rowk + colB,
                          sl);
            }
            if (VP)
              tma_load_3d(dst + NSL * PANEL_BYTES + NSL * HPANEL_BYTES, &tmB, fb, 0, rowk + colB,
                          NSL);  // V
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      if (!ok || *abort_flag) {  // drain copies in flight before the CTA can exit
        for (int s = 0; s < NSTAGE; ++s) {
          if (armed[s] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_test(full0 + 8 * s, (uint32_t)armed[s]) && clock64() - t0 < WAIT_BUDGET) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer --------------------------------
    if (lane == 0) {
      constexpr uint32_t idesc = (IDESC & ~(0x3Fu << 17)) | ((uint32_t)(HALF >> 3) << 17);
      // N = 128: the two adjacent 64-row B panels [S0b; R1b] at once
      constexpr uint32_t idesc2 = IDESC;
      int stage = 0, islot = 0;
      uint32_t phase = 0, iphase = 0;
      bool ok = true;
      uint32_t used = 0, par = 0;  // per tile: committed before / commit count parity
      while (ok) {
        if (!mbar_wait(ifull0 + 8 * islot, iphase, abort_flag, P.err, 6)) break;
        const long long qidx = item_q[islot];
        mbar_arrive(iempty0 + 8 * islot);
        if (++islot == IQ) {
          islot = 0;
          iphase ^= 1;
        }
        if (qidx < 0) break;
        int i, j, tA, tB, h;
        eos_decode(P, qidx, i, j, tA, tB, h);
        const bool same = (i == j);
        for (int o = 0; o < 4 && ok; ++o) {
          const int t = ((o & 1) << 1) | (o >> 1);
          if (same && (t & 1)) continue;
          // the tile's previous accumulators must have been read out
          if (((used >> t) & 1) &&
              !mbar_wait(tempty0 + 8 * t, ((par >> t) & 1) ^ 1u, abort_flag, P.err, 2)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dL0 = tmem + (uint32_t)(t * 2 * HALF);
          const uint32_t dL1 = dL0 + HALF;
          for (int kc = 0; kc < P.nks; ++kc) {
            if (!mbar_wait(full0 + 8 * stage, phase, abort_flag, P.err, 3)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sb = smem_u32(stages + stage * STAGE_BYTES);
            const uint32_t sbB = sb + NSL * PANEL_BYTES;
#pragma unroll
            for (int k16 = 0; k16 < KSTEP / 16; ++k16) {
              const uint32_t koff = k16 * 32;
              const uint64_t a0 = smem_desc(sb + 0 * PANEL_BYTES + koff);
              const uint64_t a1 = smem_desc(sb + 1 * PANEL_BYTES + koff);
              const uint64_t b0 = smem_desc(sbB + 0 * HPANEL_BYTES + koff);
              const uint64_t b1 = smem_desc(sbB + 1 * HPANEL_BYTES + koff);
              const uint32_t acc = (kc > 0 || k16 > 0) ? 1u : 0u;
              // [L0 | L1] += S0a x [S0b; R1b]: exact integer part and S0a R1b
              mma_f16_id(dL0, a0, b0, idesc2, acc);
              if (VP) {  // R1a V (= R1a S0b + R1a R1b + R1a eps)
                mma_f16_id(dL1, a1, smem_desc(sbB + NSL * HPANEL_BYTES + koff), idesc, 1u);
                continue;
              }
              mma_f16_id(dL1, a1, b0, idesc, 1u);   // R1a S0b
              mma_f16_id(dL1, a1, b1, idesc, 1u);   // R1a R1b
              if (NSL > 2) {
                const uint64_t a2 = smem_desc(sb + 2 * PANEL_BYTES + koff);
                const uint64_t b2 = smem_desc(sbB + 2 * HPANEL_BYTES + koff);
                mma_f16_id(dL1, a0, b2, idesc, 1u);  // S0a R2b
                mma_f16_id(dL1, a2, b0, idesc, 1u);  // R2a S0b
              }
            }
            mma_commit(empty0 + 8 * stage);
            if (++stage == NSTAGE) {
              stage = 0;
              phase ^= 1;
            }
          }
          if (!ok) break;
          mma_commit(tfull0 + 8 * t);  // tile t of this item is complete
          used |= 1u << t;
          par ^= 1u << t;
        }
      }
      // drain: all MMAs issued by this thread complete before TMEM is freed
      mma_commit(drain);
      const long long t0 = clock64();
      while (!mbar_test(drain, 0) && clock64() - t0 < WAIT_BUDGET) {
      }
    }
  } else {
    // ------------------------------ epilogue ----------------------------------
    // T1 and U1 are read into registers and released first, so the next
    // item's T1/U1 MMAs overlap this item's T2/U2 phase.
    const int ew = warp - 2;             // 0..7
    const int quad = warp & 3;
    const int cbase = (ew >> 2) * 32;    // 32 of the tile's 64 columns
    const int row = quad * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    const uint32_t tbase = tmem + lane_off + cbase;
    int islot = 0;
    uint32_t iphase = 0;
    uint32_t par = 0;  // per tile: parity of the reads so far
    bool ok = true;
    while (ok) {
      const bool w0 = mbar_wait(ifull0 + 8 * islot, iphase, abort_flag, P.err, 7);
      if (epi_any(!w0)) break;
      const long long qidx = item_q[islot];
      __syncwarp();
      if (lane == 0) mbar_arrive(iempty0 + 8 * islot);
      if (++islot == IQ) {
        islot = 0;
        iphase ^= 1;
      }
      if (qidx < 0) break;
      int i, j, tA, tB, h;
      eos_decode(P, qidx, i, j, tA, tB, h);
      const bool same = (i == j), diag = (tA == tB);
      const int a = tA * TILE + row;
      const int b0 = tB * TILE + h * HALF + cbase;
      const float *sc = P.inv, *st = P.inv + P.ncol;
      const float sCi = sc[i * P.nvpad + a], sCj = sc[j * P.nvpad + a];
      const float sTi = st[i * P.nvpad + a], sTj = st[j * P.nvpad + a];
      const float2 ea = P.ev2[a];
      const float2 ei = P.eo2[i], ej = P.eo2[j];
      const float sh = ei.x + ej.x;
      const float bv = sh - ei.x;
      const float sl = (ei.x - (sh - bv)) + (ej.x - bv) + ei.y + ej.y;
      const float dh0 = sh - ea.x;
      const float bw = dh0 - sh;
      const float dl0 = ((sh - (dh0 - bw)) + (-ea.x - bw)) + (sl - ea.y);
      // one tile's 32 columns of this thread into registers, then release it
      // g_ii(a,a) and gt_ii(a,a) of the one-residual (V plane) form carry the
      // same-column bias sum_k R1 (V - S0 - R1): its column among the
      // thread's 32 (or -1) and the two corrections, removed as T1/U1 are read
      const int cd = (VP && same && diag && a - b0 >= 0 && a - b0 < 32) ? a - b0 : -1;
      const float cg = cd >= 0 ? P.dcorr[i * P.nvpad + a] : 0.0f;
      const float cu = cd >= 0 ? P.dcorr[P.ncol + i * P.nvpad + a] : 0.0f;
      auto take = [&](int t, const float *sr, float srow, float (&v)[32]) -> bool {
        const bool w = mbar_wait(tfull0 + 8 * t, (par >> t) & 1, abort_flag, P.err, 4);
        if (epi_any(!w)) return false;
        tc_fence_after();
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
          float l0[16], l1[16];
          tmem_ld16(tbase + t * 2 * HALF + c0, l0);
          tmem_ld16(tbase + t * 2 * HALF + HALF + c0, l1);
          tmem_wait_ld();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            float x = l0[k] + l1[k];
            if (t == 0 && c0 + k == cd) x -= cg;
            if (t == 2 && c0 + k == cd) x -= cu;
            v[c0 + k] = x * (srow * sr[b0 + c0 + k]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tempty0 + 8 * t);
        par ^= 1u << t;
        return true;
      };
      float g1[32], u1[32];
      if (!take(0, sc + j * P.nvpad, sCi, g1) || !take(2, st + j * P.nvpad, sTi, u1)) {
        ok = false;
        break;
      }

      double eacc = 0.0;
      if (same) {
        float ef = 0.0f;
#pragma unroll
        for (int k = 0; k < 32; ++k) {
          const float2 eb = P.ev2[b0 + k];
          const float dh = dh0 - eb.x;
          const float bz = dh - dh0;
          const float d = dh + (((dh0 - (dh - bz)) + (-eb.x - bz)) + (dl0 - eb.y));
          // g2 = g1, u2 = u1: diagonal g1 u1, otherwise 2 g1 u1
          ef = fmaf((diag ? 1.0f : 2.0f) * g1[k] * u1[k], rcp_denom(d), ef);
        }
        eacc = (double)ef;
      } else {
        float g2[32], u2[32];
        if (!take(1, sc + i * P.nvpad, sCj, g2) || !take(3, st + i * P.nvpad, sTj, u2)) {
          ok = false;
          break;
        }
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
          float ef = 0.0f;
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const float2 eb = P.ev2[b0 + c0 + k];
            const float dh = dh0 - eb.x;
            const float bz = dh - dh0;
            const float d = dh + (((dh0 - (dh - bz)) + (-eb.x - bz)) + (dl0 - eb.y));
            const int c = c0 + k;
            float num = g1[c] * fmaf(2.0f, u1[c], -u2[c]);
            if (!diag) num = fmaf(g2[c], fmaf(2.0f, u2[c], -u1[c]), num);
            ef = fmaf(num, rcp_denom(d), ef);
          }
          eacc += (double)ef;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) eacc += __shfl_xor_sync(0xffffffffu, eacc, o);
      if (lane == 0) redd[ew] = eacc;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (ew == 0 && lane == 0) {
        double tot = 0.0;
#pragma unroll
        for (int w = 0; w < NEPI; ++w) tot += redd[w];
        P.part[qidx] = tot;
      }
      asm volatile("bar.sync 1, 256;" ::: "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

int eos_smem_bytes(int nsl, int nstage) {
  return nstage * eos_stage_bytes(nsl) + 1024 + 512;
}

// Self-test of the bounded-wait path: one thread waits on an mbarrier that
// nothing ever completes, with a short clock budget.  The wait must give up,
// raise the CTA abort flag and record `code` in the device error word, and
// the kernel must return normally.
__global__ void wait_selftest_kernel(long long budget, int *err) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool ok = mbar_wait(smem_u32(&bar), 0, (volatile int *)&abort_flag, err, 99, budget);
    if (ok) atomicCAS(err, 0, 98);  // cannot happen: nothing arrives
  }
  __syncthreads();
}

// Self-test of the epilogue's reciprocal: rcp_denom(d) beside CUDA's
// correctly rounded single-precision reciprocal __frcp_rn(d).
__global__ void rcp_selftest_kernel(const float *__restrict__ d, float *__restrict__ r,
                                    float *__restrict__ ref, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  r[t] = rcp_denom(d[t]);
  ref[t] = __frcp_rn(d[t]);
}

// --------------------------------------------------------------------------
// reductions of a batch (deterministic, compensated)
// --------------------------------------------------------------------------
__device__ __forceinline__ void two_sum_d(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void warp_sum_comp_d(double &s, double &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c, o);
    double t, e;
    if ((threadIdx.x & o) == 0)
      two_sum_d(s, s2, t, e);
    else
      two_sum_d(s2, s, t, e);
    s = t;
    c = ((threadIdx.x & o) == 0 ? c + c2 : c2 + c) + e;
  }
}

// one warp per (fragment, pair): Epair_f(i,j) = Epair_f(j,i) = sum of its items
__global__ void pair_reduce_batch_kernel(const FragDesc *__restrict__ fr, int nfrag,
                                         int npairs_total, const double *__restrict__ part) {
  const int gp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gp >= npairs_total) return;
  int lo = 0, hi = nfrag - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (fr[mid].pair_base <= gp)
      lo = mid;
    else
      hi = mid - 1;
  }
  const FragDesc &F = fr[lo];
  const int p = gp - F.pair_base;
  const double *src = part + F.item_base + (long long)p * F.ntp;
  double s = 0.0, c = 0.0;
  for (int r = lane; r < F.ntp; r += 32) {
    double t, e;
    two_sum_d(s, src[r], t, e);
    s = t;
    c += e;
  }
  warp_sum_comp_d(s, c);
  if (lane == 0) {
    int i, j;
    decode_pair(p, i, j);
    const double v = s + c;
    F.Epair[i + (size_t)F.nocc * j] = v;
    F.Epair[j + (size_t)F.nocc * i] = v;
  }
}

// one block per fragment: Etot_f = sum_ij Epair_f(i,j)
__global__ void total_reduce_batch_kernel(const FragDesc *__restrict__ fr) {
  const FragDesc &F = fr[blockIdx.x];
  __shared__ double ss[32], sc[32];
  double s = 0.0, c = 0.0;
  const size_t n = (size_t)F.nocc * F.nocc;
  for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
    double t, e;
    two_sum_d(s, F.Epair[k], t, e);
    s = t;
    c += e;
  }
  warp_sum_comp_d(s, c);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    ss[w] = s;
    sc[w] = c;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    s = lane < nw ? ss[lane] : 0.0;
    c = lane < nw ? sc[lane] : 0.0;
    warp_sum_comp_d(s, c);
    if (lane == 0) *F.Etot = s + c;
  }
}

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

int smem_bytes(int nsl, int nstage) {
  return nstage * nsl * 2 * PANEL_BYTES + 1024 /*align*/ + 512 /*barriers, ring, etc*/ +
         64 * TP * 4 /*diagonal-tile transpose buffer*/;
}

// One launch group of a batch: its fragments share a slice count and an
// energy kernel (one-CTA or paired), a slices buffer, the tensor maps and one
// persistent launch.
struct Group {
  int nsl = 2;
  int nfrag = 0;
  std::vector<FragDesc> fh;
  long long nitems = 0, R = 0, ncol_total = 0;
  int npairs_total = 0, max_ncol = 0, max_nv = 0;
  DevBuf frags, items, slices, inv, eo2, ev2, part, queue;
  CUtensorMap tm;
  // paired-CTA kernel (one residual slice): its pair items and B-half map
  bool pair = false;
  long long npitems = 0;
  DevBuf pitems, dcorr;  // dcorr: per-column diagonal correction of the V product
  CUtensorMap tmB;
  int pair_nstage = 3;  // 3: exchange transpose in shared memory; 4: through xbuf
  DevBuf xbuf;          // 4-stage form: one 64 KB exchange tile per CTA
};

// Launch with the device's highest scheduling priority.  The persistent
// energy kernels of a batch graph run beside the slicing of the next launch
// group on a side branch; without priority the slicer's many small blocks,
// ready at the same moment, fill the SMs first and the energy kernel's CTAs
// wait for them to drain.  (The priority is recorded into graph nodes.)
int energy_priority() {
  static int prio = 1;
  if (prio == 1) {
    int least = 0, greatest = 0;
    prio = cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess ? greatest : 0;
  }
  return prio;
}

template <typename... KArgs, typename... Args>
cudaError_t launch_hi(void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem,
                      cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = energy_priority();
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// Stage count of the paired kernel for a group.  The fourth 56 KB stage
// (which needs the exchange tile transposed through global scratch instead
// of shared memory) covers the cross-CTA refill round trip on long product
// chains, but measured on GB300 it gains nothing where it matters: the
// nocc=128 nvirt=1024 NBA=4096 fragment takes 5% fewer cycles at the same
// time (the power cap lowers the clock), and the 256-fragment batch runs 6%
// slower (569-572 against 605-608 eff TFLOP/s, same box: the slower
// global-memory transpose is exposed on short items).  So three stages;
// RIMP2_PAIR_STAGES=4 in the environment selects the four-stage form.
int pair_stages_for(const std::vector<FragDesc> &fh) {
  (void)fh;
  const char *e = getenv("RIMP2_PAIR_STAGES");
  if (e && e[0] == '4') return 4;
  return 3;
}

int launch_pair(const Group &g, PairParams Q, int npair, cudaStream_t s) {
  Q.xbuf = g.xbuf.as<float>();
  cudaError_t e;
  if (g.pair_nstage == 4)
    e = launch_hi(split_pair_kernel<4, true>, 2 * npair, NTHREADS, pair_smem_bytes(4, true), s,
                  g.tm, g.tmB, Q);
  else
    e = launch_hi(split_pair_kernel<3, false>, 2 * npair, NTHREADS, pair_smem_bytes(3, false),
                  s, g.tm, g.tmB, Q);
  if (e != cudaSuccess) {
    set_error("paired energy kernel launch failed: %s", cudaGetErrorString(e));
    return RIMP2_ERR_CUDA;
  }
  return RIMP2_OK;
}

int build_group(Group &g, cudaStream_t s) {
  // heaviest fragments first: their items lead the queue
  std::stable_sort(g.fh.begin(), g.fh.end(),
                   [](const FragDesc &x, const FragDesc &y) { return x.nks > y.nks; });
  long long row = 0, col = 0, item = 0, pitem = 0;
  int eo = 0, ev = 0, pb = 0;
  for (auto &F : g.fh) {
    F.nvpad = (F.nvirt + TILE - 1) / TILE * TILE;
    F.nks = (F.NBA + KSTEP - 1) / KSTEP;
    const int nt = F.nvpad / TILE;
    F.ntp = nt * (nt + 1) / 2;
    F.ncol = F.nocc * F.nvpad;
    F.eo_off = eo;
    F.ev_off = ev;
    F.pair_base = pb;
    F.row_base = row;
    F.col_base = col;
    F.item_base = item;
    F.pitem_base = pitem;
    pitem += pair_items_before(F.nocc) * F.ntp;
    const int np = F.nocc * (F.nocc + 1) / 2;
    eo += F.nocc;
    ev += F.nvpad;
    pb += np;
    row += (long long)F.nks * F.ncol;
    col += F.ncol;
    item += (long long)np * F.ntp;
    g.max_ncol = std::max(g.max_ncol, F.ncol);
    g.max_nv = std::max(g.max_nv, std::max(F.nvpad, F.nocc));
  }
  g.nfrag = (int)g.fh.size();
  g.nitems = item;
  g.npitems = pitem;
  g.R = row;
  g.ncol_total = col;
  g.npairs_total = pb;
  if (g.R > 2147483647LL - TILE || g.nitems > 2147483647LL) {
    set_error("split batch too large for one launch (rows=%lld, items=%lld)", g.R, g.nitems);
    return RIMP2_ERR_ARG;
  }
  if (g.pair && g.npitems > 2147483647LL) {
    set_error("split batch too large for one launch (pair items=%lld)", g.npitems);
    return RIMP2_ERR_ARG;
  }
  const int planes = g.nsl + (g.pair ? 1 : 0);  // the paired kernel adds the V plane
  RIMP2_TRY(g.frags.alloc(sizeof(FragDesc) * g.nfrag, s));
  RIMP2_TRY(g.items.alloc(sizeof(int4) * (size_t)g.nitems, s));
  RIMP2_TRY(g.slices.alloc(sizeof(__half) * (size_t)planes * (size_t)g.R * 64, s));
  RIMP2_TRY(g.inv.alloc(sizeof(float) * (size_t)g.ncol_total, s));
  if (g.pair) RIMP2_TRY(g.dcorr.alloc(sizeof(float) * (size_t)g.ncol_total, s));
  RIMP2_TRY(g.eo2.alloc(sizeof(float2) * (size_t)eo, s));
  RIMP2_TRY(g.ev2.alloc(sizeof(float2) * (size_t)ev, s));
  RIMP2_TRY(g.part.alloc(sizeof(double) * (size_t)g.nitems, s));
  RIMP2_TRY(g.queue.alloc(sizeof(unsigned int), s));
  RIMP2_CK(cudaMemcpyAsync(g.frags.p, g.fh.data(), sizeof(FragDesc) * g.nfrag,
                           cudaMemcpyHostToDevice, s));
  build_items_kernel<<<(unsigned)((g.nitems + 255) / 256), 256, 0, s>>>(
      g.frags.as<FragDesc>(), g.nfrag, g.nitems, g.items.as<int4>());
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  auto encode = get_encode();
  if (!encode) {
    set_error("cuTensorMapEncodeTiled entry point unavailable");
    return RIMP2_ERR_UNSUPPORTED;
  }
  cuuint64_t dims[3] = {64, (cuuint64_t)g.R, (cuuint64_t)planes};
  cuuint64_t strides[2] = {128, (cuuint64_t)g.R * 128};
  cuuint32_t box[3] = {KSTEP, TILE, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult cr = encode(&g.tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, g.slices.p, dims, strides, box,
                       estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return RIMP2_ERR_CUDA;
  }
  auto k2 = split_batch_kernel<2, 3>;
  auto k3 = split_batch_kernel<3, 2>;
  RIMP2_CK(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(2, 3)));
  RIMP2_CK(cudaFuncSetAttribute(k3, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes(3, 2)));
  if (g.pair) {
    g.pair_nstage = pair_stages_for(g.fh);
    if (g.pair_nstage == 4) {
      int dev = 0, nsm = 0;
      RIMP2_CK(cudaGetDevice(&dev));
      RIMP2_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      RIMP2_TRY(g.xbuf.alloc(sizeof(float) * TILE * TILE * (size_t)nsm, s));
      RIMP2_CK(cudaFuncSetAttribute(split_pair_kernel<4, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    pair_smem_bytes(4, true)));
    } else {
      RIMP2_CK(cudaFuncSetAttribute(split_pair_kernel<3, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    pair_smem_bytes(3, false)));
    }
    cuuint32_t boxB[3] = {KSTEP, BHALF, 1};
    cr = encode(&g.tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, g.slices.p, dims, strides, boxB, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
      return RIMP2_ERR_CUDA;
    }
    RIMP2_TRY(g.pitems.alloc(sizeof(int4) * (size_t)g.npitems, s));
    build_pair_items_kernel<<<(unsigned)((g.npitems + 255) / 256), 256, 0, s>>>(
        g.frags.as<FragDesc>(), g.nfrag, g.npitems, g.pitems.as<int4>());
    count_launch(1);
    RIMP2_CK(cudaGetLastError());
  }
  return RIMP2_OK;
}

// The group's inputs for its energy kernel: slices, scales, corrections and
// orbital-energy pairs (graph-capturable: no sync, no alloc).
int record_group_inputs(Group &g, cudaStream_t s) {
  if (g.nfrag == 0) return RIMP2_OK;
  const FragDesc *fr = g.frags.as<FragDesc>();
  dim3 grid((unsigned)((g.max_ncol * 32LL + 255) / 256), (unsigned)g.nfrag);
  slice_batch_kernel<<<grid, 256, 0, s>>>(fr, g.nsl, g.R * 64, g.slices.as<__half>(),
                                          g.inv.as<float>(), 0, 0x7fffffff, g.pair ? 1 : 0,
                                          g.dcorr.as<float>());
  dim3 g2((unsigned)((g.max_nv + 255) / 256), (unsigned)g.nfrag);
  eps_batch_kernel<<<g2, 256, 0, s>>>(fr, g.eo2.as<float2>(), g.ev2.as<float2>());
  count_launch(2);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

// Enqueue one evaluation of the group on s (graph-capturable: no sync, no
// alloc); with_inputs = false when its inputs were enqueued elsewhere.
int record_group(Group &g, cudaStream_t s, int nsm, cudaEvent_t *ev /* 3 or null */,
                 bool with_inputs = true) {
  if (g.nfrag == 0) return RIMP2_OK;
  const FragDesc *fr = g.frags.as<FragDesc>();
  if (ev) RIMP2_CK(cudaEventRecord(ev[0], s));
  if (with_inputs) RIMP2_TRY(record_group_inputs(g, s));
  RIMP2_CK(cudaMemsetAsync(g.queue.p, 0, sizeof(unsigned int), s));
  BatchParams P;
  P.frags = fr;
  P.items = g.items.as<int4>();
  P.nitems = g.nitems;
  P.item_begin = 0;
  P.queue = g.queue.as<unsigned int>();
  P.eo2 = g.eo2.as<float2>();
  P.ev2 = g.ev2.as<float2>();
  P.inv_scale = g.inv.as<float>();
  P.part = g.part.as<double>();
  P.err = device_error_word();
  const int grid = (int)std::min<long long>(g.nitems, nsm);
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  if (ev) RIMP2_CK(cudaEventRecord(ev[1], s));
  if (g.pair) {
    PairParams Q;
    Q.frags = fr;
    Q.items = g.pitems.as<int4>();
    Q.nitems = g.npitems;
    Q.item_begin = 0;
    Q.dcorr = g.dcorr.as<float>();
    Q.queue = P.queue;
    Q.eo2 = P.eo2;
    Q.ev2 = P.ev2;
    Q.inv_scale = P.inv_scale;
    Q.part = P.part;
    Q.err = P.err;
    const int npair = (int)std::min<long long>(g.npitems, std::max(1, nsm / 2));
    RIMP2_TRY(launch_pair(g, Q, npair, s));
    note_split_kernel(2);
  } else if (g.nsl == 2) {
    note_split_kernel(1);
    RIMP2_CK(launch_hi(split_batch_kernel<2, 3>, grid, BATCH_THREADS, smem_bytes(2, 3), s, g.tm, P));
  } else {
    note_split_kernel(1);
    RIMP2_CK(launch_hi(split_batch_kernel<3, 2>, grid, BATCH_THREADS, smem_bytes(3, 2), s, g.tm, P));
  }
  count_launch(1);
  if (ev) RIMP2_CK(cudaEventRecord(ev[2], s));
  pair_reduce_batch_kernel<<<(unsigned)((g.npairs_total + 7) / 8), 256, 0, s>>>(
      fr, g.nfrag, g.npairs_total, g.part.as<double>());
  total_reduce_batch_kernel<<<g.nfrag, 1024, 0, s>>>(fr);
  count_launch(2);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

// ==========================================================================
// General split-precision GEMM on the same slices (used by the AO->MO
// transform): D[m][n] = sum_k A[m][k] B[n][k], A and B K-major FP16 slices
// with per-row power-of-two scales, exact integer L0 + residual L1 in TMEM,
// FP64 output (L0 and L1 combined in FP64) with arbitrary strides.
// Persistent: each CTA takes output tiles (128 x NT, NT <= 128) blockIdx.x,
// + gridDim.x, ... (all tiles have the same K), with two TMEM accumulator
// sets, so that the epilogue of one tile (TMEM -> FP64 stores) runs while
// the tensor core works on the next and the copy ring never drains between
// tiles.  Per K16 step one MMA over the stacked B planes [S0b; R1b] (N = 2 NT)
// gives L0 and S0a R1b, then R1a S0b, R1a R1b (and S0a R2b, R2a S0b with two
// residual slices) accumulate into L1.
// Roles: warp 0 TMA producer, warp 1 MMA issuer and TMEM owner, warps 2-9
// epilogue (two per TMEM lane quadrant, alternate 16-column chunks).  Every
// wait is bounded.
// ==========================================================================
struct GemmSP {
  int M, N, NT, nks, mtiles, ntiles, nbatch;
  long long a_ncol, b_ncol;        // rows per K chunk in each operand's slice layout
  long long a_row0, a_bstride;     // first row of batch 0 and row stride between batches
  long long b_row0, b_bstride;
  const float *a_inv, *b_inv;      // per-row inverse scales (indexed like the rows)
  double *out;
  long long sOm, sOn, sOb;
  uint32_t tmem_cols;              // TMEM columns allocated (a power of two >= 4 NT)
  int *err;
};

constexpr int GEMM_NST = 2;

constexpr int gemm_stage_bytes(int nsl, int NT) { return nsl * (PANEL_BYTES + NT * 128); }
constexpr int gemm_smem_bytes(int nsl, int NT) {
  return GEMM_NST * gemm_stage_bytes(nsl, NT) + 1024 + 256;
}

constexpr int GEMM_EPI = 8;                       // epilogue warps: two per lane quadrant
constexpr int GEMM_THREADS = 64 + 32 * GEMM_EPI;

template <int NSL>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    split_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      GemmSP P) {
  constexpr int NST = GEMM_NST;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int NT = P.NT;
  const int BPL = NT * 128;  // bytes of one B plane (NT rows of 64 FP16)
  const int STAGE = NSL * (PANEL_BYTES + BPL);
  // bars: full[2], empty[2], tfull[2], tempty[2], drain
  uint64_t *bars = (uint64_t *)(base + NST * STAGE);
  uint32_t *tmem_slot = (uint32_t *)(bars + 2 * NST + 5);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(&bars[0]), empty0 = smem_u32(&bars[NST]);
  const uint32_t tfull0 = smem_u32(&bars[2 * NST]), tempty0 = smem_u32(&bars[2 * NST + 2]);
  const uint32_t drain = smem_u32(&bars[2 * NST + 4]);
  const long long per_b = (long long)P.mtiles * P.ntiles;
  const long long nitems = per_b * P.nbatch;
  if (threadIdx.x == 0) {
    for (int st = 0; st < NST; ++st) {
      mbar_init(full0 + 8 * st, 1);
      mbar_init(empty0 + 8 * st, 1);
    }
    for (int u = 0; u < 2; ++u) {
      mbar_init(tfull0 + 8 * u, 1);
      mbar_init(tempty0 + 8 * u, GEMM_EPI);  // the epilogue warps
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(P.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto tile_rows = [&](long long item, long long &arow, long long &brow, int &b, int &mt, int &nt) {
    b = (int)(item / per_b);
    const long long rem = item % per_b;
    mt = (int)(rem / P.ntiles);
    nt = (int)(rem % P.ntiles);
    arow = P.a_row0 + (long long)b * P.a_bstride + (long long)mt * TILE;
    brow = P.b_row0 + (long long)b * P.b_bstride + (long long)nt * NT;
  };
  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int armed[NST] = {-1, -1};
      bool ok = true;
      const uint32_t tx = (uint32_t)STAGE;
      for (long long item = blockIdx.x; item < nitems && ok; item += gridDim.x) {
        long long arow, brow;
        int b, mt, nt;
        tile_rows(item, arow, brow, b, mt, nt);
        for (int kc = 0; kc < P.nks; ++kc) {
          if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag, P.err, 11)) {
            ok = false;
            break;
          }
          const uint32_t fb = full0 + 8 * stage;
          mbar_expect_tx(fb, tx);
          armed[stage] = (int)phase;
          const uint32_t dst = smem_u32(base + stage * STAGE);
#pragma unroll
          for (int sl = 0; sl < NSL; ++sl) {  // A planes, then the B planes back to back
            tma_load_3d(dst + sl * PANEL_BYTES, &tmA, fb, 0, (int)(kc * P.a_ncol + arow), sl);
            tma_load_3d(dst + NSL * PANEL_BYTES + sl * BPL, &tmB, fb, 0,
                        (int)(kc * P.b_ncol + brow), sl);
          }
          if (++stage == NST) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      if (!ok || *abort_flag) {  // copies in flight land before the CTA can exit
        for (int st = 0; st < NST; ++st) {
          if (armed[st] < 0) continue;
          const long long t0 = clock64();
          while (!mbar_test(full0 + 8 * st, (uint32_t)armed[st]) && clock64() - t0 < WAIT_BUDGET) {
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer --------------------------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true;
      const uint32_t id2 = idesc_mn(TILE, 2 * NT), id1 = idesc_mn(TILE, NT);
      long long t = 0;  // tiles of this CTA so far
      for (long long item = blockIdx.x; item < nitems && ok; item += gridDim.x, ++t) {
        const int u = (int)(t & 1);
        // the epilogue has read this accumulator set's previous tile
        if (t >= 2 &&
            !mbar_wait(tempty0 + 8 * u, (uint32_t)(((t >> 1) - 1) & 1), abort_flag, P.err, 14)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t dL0 = tmem + (uint32_t)(u * 2 * NT), dL1 = dL0 + (uint32_t)NT;
        for (int kc = 0; kc < P.nks; ++kc) {
          if (!mbar_wait(full0 + 8 * stage, phase, abort_flag, P.err, 12)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(base + stage * STAGE);
          const uint32_t sb = sa + NSL * PANEL_BYTES;
#pragma unroll
          for (int k16 = 0; k16 < KSTEP / 16; ++k16) {
            const uint32_t koff = k16 * 32;
            const uint64_t a0 = smem_desc(sa + koff), a1 = smem_desc(sa + PANEL_BYTES + koff);
            const uint64_t b0 = smem_desc(sb + koff), b1 = smem_desc(sb + BPL + koff);
            const uint32_t acc = (kc > 0 || k16 > 0) ? 1u : 0u;
            mma_f16_id(dL0, a0, b0, id2, acc);  // [L0 | L1] = S0a [S0b; R1b]
            mma_f16_id(dL1, a1, b0, id1, 1u);   // R1a S0b
            mma_f16_id(dL1, a1, b1, id1, 1u);   // R1a R1b
            if (NSL > 2) {
              const uint64_t a2 = smem_desc(sa + 2 * PANEL_BYTES + koff);
              const uint64_t b2 = smem_desc(sb + 2 * BPL + koff);
              mma_f16_id(dL1, a0, b2, id1, 1u);  // S0a R2b
              mma_f16_id(dL1, a2, b0, id1, 1u);  // R2a S0b
            }
          }
          mma_commit(empty0 + 8 * stage);
          if (++stage == NST) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        mma_commit(tfull0 + 8 * u);
      }
      mma_commit(drain);
      const long long t0 = clock64();
      while (!mbar_test(drain, 0) && clock64() - t0 < WAIT_BUDGET) {
      }
    }
  } else {
    // ------------------------------ epilogue ----------------------------------
    const int quad = warp & 3;
    const int half = (warp - 2) >> 2;  // 16-column chunks half, half + 2, ...
    const int row = quad * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    long long t = 0;
    for (long long item = blockIdx.x; item < nitems; item += gridDim.x, ++t) {
      const int u = (int)(t & 1);
      if (!mbar_wait(tfull0 + 8 * u, (uint32_t)((t >> 1) & 1), abort_flag, P.err, 13)) break;
      tc_fence_after();
      long long arow, brow;
      int b, mt, nt;
      tile_rows(item, arow, brow, b, mt, nt);
      const long long m = (long long)mt * TILE + row;
      const float sa = P.a_inv[arow + row];  // 2^-e of this row
      const uint32_t taddr = tmem + lane_off + (uint32_t)(u * 2 * NT);
      double *orow = P.out + (long long)b * P.sOb + m * P.sOm;
      for (int c0 = 16 * half; c0 < NT; c0 += 32) {
        float l0[16], l1[16];
        tmem_ld16(taddr + c0, l0);
        tmem_ld16(taddr + NT + c0, l1);
        tmem_wait_ld();
        if (m < P.M) {
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int n = nt * NT + c0 + k;
            if (n < P.N) {
              // (L0 + L1) sa sb with one FP64 operation: L0 (an integer
              // below 2^24) and L1 times the row's power of two are exact
              // floats (|L1 sa| below 2^-126, far under the output's
              // resolution, flushes), their sum rounds once in FP64 as
              // (L0 + L1) does, and the column's power of two moves the
              // exponent.  The FP64 pipe, not the tensor core, bounded this
              // epilogue with FP64 conversions and products per element.
              const double v = f2d_bits(l0[k] * sa) + f2d_bits(l1[k] * sa);
              orow[(long long)n * P.sOn] = scale_pow2(v, P.b_inv[brow + c0 + k]);
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty0 + 8 * u);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(P.tmem_cols)
                 : "memory");
  }
}

// ==========================================================================
// Fused first half of the AO->MO transform on the tensor cores, one pass over
// the FP64 AO tensor:  H[i][alpha][mu] = sum_nu (alpha|mu nu) Cmo(nu, i),
// evaluated as sum_nu (alpha|nu mu) Cmo(nu, i): the three-centre integrals
// are symmetric in their two AO indices, and the middle one is the short
// stride (8 NBA bytes), so every 64-value chunk of a row lies in one memory
// page (the last index is 8 NBA nbas bytes apart: a chunk would touch 64).
// GEMM rows are (alpha, mu) -- 16 alpha x 8 mu per CTA tile, row r = a + 16 m
// -- K = nu in chunks of 64, N = the occupied orbitals (NT <= 80, padded to
// a multiple of 16).  The AO tensor is read once -- per row group (the 32
// rows of 16 alpha x 2 mu) one 16 alpha x 64 nu x 2 mu TMA box per chunk
// (even NBA, 16-byte aligned tensor), or per-thread 8-byte cp.async copies
// otherwise -- and sliced by the converter warps (an FP32-arithmetic split,
// split_f32) with a power-of-two scale per (row, K chunk):
// |x 2^e| <= 511.5, so S0 is a 10-bit integer, and with the occupied MO
// block sliced the same way (per column and chunk, precomputed) every
// partial sum of S0a S0b over a chunk is below 64 * 511^2 < 2^24: the integer
// part of each chunk's product is exact in FP32.  Products per element pair:
// S0 S0 (L0), S0 R1 + R1 S0 + R1 R1 + S0 R2 + R2 S0 (L1).  Each chunk's L0/L1
// go to one of two TMEM buffers; the epilogue scales them by the row and
// column scales of that chunk (powers of two: exact) and adds them into a
// double-float (FP32 hi + lo, two-sum) running total kept in TMEM, so the
// result carries ~2^-40 of the chunk products' magnitude.  At the end of
// the tile the totals are converted to FP64 (bits moved, one FP64 add: the
// FP64 pipe is slow on GB300), staged in shared memory and written as
// 64-byte runs of 8 mu per (i, alpha).
// Roles: warps 0-15 converters (row r = 32 (w & 3) + lane, K quarter w >> 2
// of each chunk: 16 values a thread), warp 16 MMA issuer and TMEM owner.
// The converter warps are also the epilogue: each is bound to the TMEM lane
// quadrant of its rows and takes a quarter of the NT columns; in iteration
// c they slice chunk c and then fold chunk c-1's accumulators into the
// running totals, while the tensor core runs chunk c.  The four warps of a
// row group synchronise among themselves only (the chunk maxima exchange),
// so the groups' latency-bound phases interleave; a group's next box is
// requested as soon as its warps hold their values (the cp.async form
// copies after the chunk is handed to the tensor core and prefetches the
// chunk after that into L2).  The converter warps bound the kernel (issue
// about 44% active; 3.11 ms at nbas=680, 6.45 ms with all 16 warps in
// lockstep, a 64-bit integer split, cp.async copies and FP64-pipe
// conversions).  Every wait is bounded; on expiry the CTA records an error
// code, drains its copies and MMAs and returns.
// --------------------------------------------------------------------------
constexpr int AH_TA = 16, AH_TM = 8;  // alpha x mu rows of a tile (16 x 8 = 128)
constexpr int AH_CONV = 16;
constexpr int AH_THREADS = 32 * (AH_CONV + 1);
constexpr int AH_NT_MAX = 80;
constexpr int AH_STG = AH_TA * 9;  // staged output doubles per column

struct AoHalfParams {
  const double *ao;   // (alpha|mu nu), alpha fastest: ao[alpha + NBA (mu + nbas nu)]
  int NBA, nbas, nocc, NT, nks;
  int ta_tiles;       // alpha tiles (of 16)
  const float *sb;    // [chunk][NT] column scales of the sliced occupied MO block
  double *half;       // H[i][alpha][mu]
  uint32_t idesc;
  int *err;
};

constexpr int ah_b_plane(int NT) { return NT * 128; }  // bytes of one B plane (NT rows x 64 FP16)
constexpr int ah_stage_bytes(int NT) { return 3 * PANEL_BYTES + 3 * ah_b_plane(NT); }
constexpr int AH_SLOT_BYTES = KSTEP * 128 * 8;  // one FP64 chunk of the tile (64 KB)
constexpr int ah_smem_bytes(int NT) {
  return 1024 + 2 * ah_stage_bytes(NT) + AH_SLOT_BYTES + 2 * 4 * 128 * 4 /*row max exchange*/ +
         2 * 128 * 4 /*row scales*/ + 256 /*barriers, slot*/;
}

// 8-byte asynchronous global -> shared copy; src_bytes = 0 fills zeros and
// reads nothing
__device__ __forceinline__ void cp_async8_zfill(uint32_t dst, const void *src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(src_bytes)
               : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_st4(uint32_t taddr, const float (&v)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3]))
               : "memory");
}

__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}

// Fold of W columns (4 or 8) of one AO chunk's products into the running
// double-float totals: L0 and L1 scaled by the row and column powers of two
// (exact), added to hi/lo with a two-sum of the high parts (first chunk:
// assigned), written back to TMEM -- or, on the last chunk, turned into
// FP64 in the staging area ([column][alpha][mu], 9-double pitch per alpha).
template <int W>
__device__ __forceinline__ void ah_fold(uint32_t tL0, int NT, uint32_t rs_hi, uint32_t rs_lo,
                                        int col, float sa, const float *sbc, bool first,
                                        bool last, double *stg, int a_l, int m_l) {
  float l0[W], l1[W], hi[W], lo[W], sbk[W];
#pragma unroll
  for (int q = 0; q < W; q += 4) {  // 16-byte loads (NT and col are multiples of 4)
    const float4 sb4 = *reinterpret_cast<const float4 *>(sbc + col + q);
    sbk[q] = sb4.x;
    sbk[q + 1] = sb4.y;
    sbk[q + 2] = sb4.z;
    sbk[q + 3] = sb4.w;
  }
  if constexpr (W == 8) {
    tmem_ld8(tL0 + col, l0);
    tmem_ld8(tL0 + NT + col, l1);
    if (!first) {
      tmem_ld8(rs_hi + col, hi);
      tmem_ld8(rs_lo + col, lo);
    }
  } else {
    tmem_ld4(tL0 + col, l0);
    tmem_ld4(tL0 + NT + col, l1);
    if (!first) {
      tmem_ld4(rs_hi + col, hi);
      tmem_ld4(rs_lo + col, lo);
    }
  }
  tmem_wait_ld();
#pragma unroll
  for (int k = 0; k < W; ++k) {
    const float sc = sa * sbk[k];  // power of two: the products below are exact
    const float xh = l0[k] * sc, xl = l1[k] * sc;
    if (first) {
      hi[k] = xh;
      lo[k] = xl;
    } else {  // two-sum of the high parts, low parts added
      const float s = hi[k] + xh;
      const float bv = s - hi[k];
      const float err = (hi[k] - (s - bv)) + (xh - bv);
      lo[k] = lo[k] + xl + err;
      hi[k] = s;
    }
  }
  if (!last) {
    if constexpr (W == 8) {
      tmem_st8(rs_hi + col, hi);
      tmem_st8(rs_lo + col, lo);
    } else {
      tmem_st4(rs_hi + col, hi);
      tmem_st4(rs_lo + col, lo);
    }
  } else {
#pragma unroll
    for (int k = 0; k < W; ++k)  // one FP64 add per output (bit-moved conversions)
      stg[(col + k) * AH_STG + a_l * 9 + m_l] = f2d_bits(hi[k]) + f2d_bits(lo[k]);
  }
}

// Exponent e with |x| 2^e <= 511.5 (to within 2^-11) for the largest
// magnitude of a row or column chunk, from key = the top 32 bits of its FP64
// pattern (11 exponent, 20 fraction bits): mx = m 2^E with m in [1, 2), and
// m <= 1.998046875 (fraction key <= 0xFFE00) allows e = 8 - E.  A value that
// shares the key but has nonzero lower bits gives |x| 2^e < 511.5003, which
// rounds to |q| <= 512: still exact in FP16, and 64 products of two such
// integers stay <= 2^24, exact in FP32.  At most 126, so that 2^-e is a
// normal float; at least -126 (|x| < 2^134); 0 for a chunk of zeros and
// subnormals.
__device__ __forceinline__ int chunk_exponent_511(uint32_t key) {
  const int ed = (int)(key >> 20);
  if (ed == 0) return 0;
  const int E = ed - 1023;
  const int e = ((key & 0xFFFFFu) <= 0xFFE00u ? 8 : 7) - E;
  return max(-126, min(126, e));
}

// Bounded vote over the converter threads (named barrier 2).
__device__ __forceinline__ bool conv_any(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, 2, %2, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(32 * AH_CONV)
      : "memory");
  return r != 0;
}

// Bounded vote over the 128 converter threads of row group g (the four warps
// that hold the same tile rows; named barrier 3 + g).
__device__ __forceinline__ bool group_any(bool p, int g) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, o;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred o, %2, 128, q;\n\t"
      "selp.u32 %0, 1, 0, o;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(3 + g)
      : "memory");
  return r != 0;
}

template <bool AO_TMA>
__global__ void __maxnreg__(96)
    ao_half_kernel(const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmAO,
                   AoHalfParams P) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int NT = P.NT;
  const int BPL = ah_b_plane(NT);
  const int STAGE = 3 * PANEL_BYTES + 3 * BPL;
  uint8_t *stages = base;
  double *slot = (double *)(base + 2 * STAGE);                     // [64 k][128 rows] FP64
  uint32_t *smx = (uint32_t *)(base + 2 * STAGE + AH_SLOT_BYTES);  // [2 parity][4 quarter][128]
  float *sscale = (float *)(smx + 2 * 4 * 128);                    // [2][128]
  uint64_t *bars = (uint64_t *)(sscale + 2 * 128);
  // bars: stage_full[2], stage_empty[2], acc_full[2], acc_empty[2], drain,
  //       ao_full[4] (the AO chunk of each row group, TMA form)
  uint32_t *tmem_slot = (uint32_t *)(bars + 13);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
  const uint32_t sfull0 = smem_u32(&bars[0]), sempty0 = smem_u32(&bars[2]);
  const uint32_t afull0 = smem_u32(&bars[4]), aempty0 = smem_u32(&bars[6]);
  const uint32_t drain = smem_u32(&bars[8]);
  const uint32_t aofull0 = smem_u32(&bars[9]);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ta = blockIdx.x % P.ta_tiles, tm = blockIdx.x / P.ta_tiles;
  const int alpha0 = ta * AH_TA, mu0 = tm * AH_TM;
  const int nks = P.nks;

  if (threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(sfull0 + 8 * b, 32 * AH_CONV);  // every converter thread (one with the B bytes)
      mbar_init(sempty0 + 8 * b, 1);            // MMA commit
      mbar_init(afull0 + 8 * b, 1);             // MMA commit
      mbar_init(aempty0 + 8 * b, AH_CONV);      // converter warps, after reading the chunk
    }
    mbar_init(drain, 1);
    for (int g = 0; g < 4; ++g) mbar_init(aofull0 + 8 * g, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
    if (AO_TMA) asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmAO) : "memory");
  }
  if (warp == AH_CONV) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < AH_CONV) {
    // ------------------------- converters and epilogue ------------------------
    const int r = 32 * (warp & 3) + lane;  // tile row = TMEM lane of this thread
    const int kq = warp >> 2;              // K quarter of each chunk; column quarter of N
    const int a_l = r % AH_TA, m_l = r / AH_TA;
    const int alpha = alpha0 + a_l, mu = mu0 + m_l;
    const bool live = alpha < P.NBA && mu < P.nbas;
    // row (alpha, mu) contracted over the middle index: (alpha|nu mu) =
    // (alpha|mu nu), and the middle index is 8 NBA bytes apart, so a chunk of
    // 64 values stays inside one memory page (the last index: 64 pages)
    const long long kstride = P.NBA;
    const double *src = P.ao + (live ? (long long)alpha + (long long)P.NBA * P.nbas * mu : 0);
    const int within = r & 7;
    int armed = -1;  // thread 0: parity of the last stage it armed for the B copy
    int armed_b = 0;
    // this thread's 16 values of a chunk in the FP64 slot: k = 16 kq + j.
    // cp.async form: [k][row]; TMA form: one 16 KB box per row group g
    // (16 alpha x 64 k x 2 mu, alpha fastest), value (a_l, k, m_l) at
    // g * 2048 + ((m_l & 1) * 64 + k) * 16 + a_l
    const int rg = warp & 3;
    double *myslot = AO_TMA ? slot + rg * 2048 + ((m_l & 1) * 64 + 16 * kq) * 16 + a_l
                            : slot + (16 * kq) * 128 + r;
    const int jstride = AO_TMA ? 16 : 128;
    const uint32_t myslot_s = smem_u32(myslot);
    const uint32_t aofull = aofull0 + 8 * rg;
    // TMA form: lane 0 of the group's K-quarter-0 warp issues the group's box
    const bool ao_issuer = AO_TMA && kq == 0 && lane == 0;
    int ao_pending = -1;  // parity of a box in flight (issuer)
    auto issue_box = [&](int c) {
      mbar_expect_tx(aofull, AH_TA * KSTEP * 2 * 8);
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
          " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(slot + rg * 2048)),
          "l"((uint64_t)&tmAO), "r"(aofull), "r"(alpha0), "r"(c * KSTEP), "r"(mu0 + 2 * rg)
          : "memory");
      ao_pending = c & 1;
    };
    // L2 prefetch of a later chunk: thread t covers the 16-alpha run (128
    // bytes, at most two lines) of k = t / 8 and mu = mu0 + t % 8, so that
    // the chunk's cp.async copies find their data in L2; with one chunk in
    // flight per CTA the copies would otherwise wait out the slowest DRAM
    // access of each chunk
    const int pf_k = threadIdx.x >> 3, pf_m = mu0 + (threadIdx.x & 7);
    const int pf_a = min(AH_TA, P.NBA - alpha0);  // alpha values of the tile
    auto prefetch_chunk = [&](int c) {
      const int k = c * KSTEP + pf_k;
      if (k < P.nbas && pf_m < P.nbas) {
        const double *p = P.ao + alpha0 + (long long)P.NBA * k + (long long)P.NBA * P.nbas * pf_m;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(p + (pf_a - 1)));
      }
    };
    auto issue_chunk = [&](int c) {
      const int k0 = c * KSTEP + 16 * kq;
      const int lim = live ? min(16, P.nbas - k0) : 0;  // values that exist
      const double *p = src + kstride * k0;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        cp_async8_zfill(myslot_s + j * 128 * 8, j < lim ? (const void *)p : (const void *)P.ao,
                        j < lim ? 8u : 0u);
        p += kstride;
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // epilogue of chunk ce: its L0/L1 scaled by the row and column scales of
    // the chunk and added to the running double-float totals (TMEM), or on
    // the last chunk turned into FP64 in the staging area
    const int ncol = NT / 4, col0 = kq * ncol;
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t rs_hi = tmem + lane_off + (uint32_t)(4 * NT);
    const uint32_t rs_lo = rs_hi + (uint32_t)NT;
    auto epilogue = [&](int ce) -> bool {
      const int b = ce & 1;
      if (!mbar_wait(afull0 + 8 * b, (uint32_t)((ce >> 1) & 1), abort_flag, P.err, 25)) return false;
      tc_fence_after();
      const float sa = sscale[b * 128 + r];
      const uint32_t tL0 = tmem + lane_off + (uint32_t)(b * 2 * NT);
      const float *sbc = P.sb + (size_t)ce * NT;
      const bool last = ce + 1 == nks;
      double *stg = reinterpret_cast<double *>(stages);
      // eight columns per TMEM round trip, four for a remainder
      int col = col0;
      for (; col + 8 <= col0 + ncol; col += 8)
        ah_fold<8>(tL0, NT, rs_hi, rs_lo, col, sa, sbc, ce == 0, last, stg, a_l, m_l);
      if (col < col0 + ncol)
        ah_fold<4>(tL0, NT, rs_hi, rs_lo, col, sa, sbc, ce == 0, last, stg, a_l, m_l);
      if (!last) tmem_wait_st();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(aempty0 + 8 * b);
      return true;
    };
    bool ok_all = true;
    if (AO_TMA) {
      if (ao_issuer) issue_box(0);
    } else {
      if (nks > 1) prefetch_chunk(1);
      issue_chunk(0);
    }
    for (int c = 0; c < nks; ++c) {
      const int b = c & 1;
      bool landed = true;
      if (AO_TMA) {
        landed = mbar_wait(aofull, (uint32_t)(c & 1), abort_flag, P.err, 26);
        if (ao_issuer && landed) ao_pending = -1;
      } else {
        if (c + 2 < nks) prefetch_chunk(c + 2);
        // chunk c has landed (each thread reads only the values it copied)
        asm volatile("cp.async.wait_group 0;" ::: "memory");
      }
      double v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) v[j] = myslot[j * jstride];
      uint32_t key = 0;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const uint32_t kj = (uint32_t)(((unsigned long long)__double_as_longlong(v[j]) >> 32) &
                                       0x7FFFFFFFu);
        key = kj > key ? kj : key;
      }
      smx[(b * 4 + kq) * 128 + r] = key;
      bool ok = landed;
      if (ok && c >= 2)
        ok = mbar_wait(sempty0 + 8 * b, (uint32_t)(((c - 2) >> 1) & 1), abort_flag, P.err, 21);
      // the four warps of a row group exchange their K quarters' maxima; the
      // groups do not wait for one another, so their latency-bound phases
      // (loads, slicing, TMEM round trips) interleave
      if (group_any(!ok, warp & 3)) {
        ok_all = false;
        break;
      }
      // every warp of the group has its values: the group's box is free
      if (ao_issuer && c + 1 < nks) issue_box(c + 1);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t o = smx[(b * 4 + q) * 128 + r];
        key = o > key ? o : key;
      }
      const int e = chunk_exponent_511(key);
      if (kq == 0) sscale[b * 128 + r] = ldexpf(1.0f, -e);
      uint8_t *st = stages + b * STAGE;
#pragma unroll
      for (int g = 0; g < 2; ++g) {
        __align__(16) __half2 h0[4], h1[4], h2[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // two values at a time, packed conversions
          float qa, ra, qb, rb;
          split_f32(v[8 * g + 2 * q], e, qa, ra);
          split_f32(v[8 * g + 2 * q + 1], e, qb, rb);
          h0[q] = __floats2half2_rn(qa, qb);  // |q| <= 512: exact in FP16
          h1[q] = __floats2half2_rn(ra, rb);
          const float2 f1 = __half22float2(h1[q]);
          h2[q] = __floats2half2_rn(ra - f1.x, rb - f1.y);
        }
        const int phys = (2 * kq + g) ^ within;  // 128-byte swizzle of 16-byte chunks
        const int off = (r >> 3) * 1024 + within * 128 + phys * 16;
        *reinterpret_cast<uint4 *>(st + 0 * PANEL_BYTES + off) = *reinterpret_cast<const uint4 *>(h0);
        *reinterpret_cast<uint4 *>(st + 1 * PANEL_BYTES + off) = *reinterpret_cast<const uint4 *>(h1);
        *reinterpret_cast<uint4 *>(st + 2 * PANEL_BYTES + off) = *reinterpret_cast<const uint4 *>(h2);
      }
      // generic-proxy writes of the A panels become visible to the tensor core
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (threadIdx.x == 0) {
        const uint32_t fb = sfull0 + 8 * b;
        mbar_expect_tx(fb, 3 * BPL);
        armed = (int)((c >> 1) & 1);
        armed_b = b;
        const uint32_t dst = smem_u32(st + 3 * PANEL_BYTES);
#pragma unroll
        for (int p = 0; p < 3; ++p) tma_load_3d(dst + p * BPL, &tmB, fb, 0, 0, 3 * c + p);
      } else {
        mbar_arrive(sfull0 + 8 * b);
      }
      // the next chunk's copies overlap the previous chunk's epilogue and
      // the next iteration's start (the L2 prefetch keeps their latency short)
      if (!AO_TMA && c + 1 < nks) issue_chunk(c + 1);
      // the previous chunk's epilogue runs while this chunk's MMAs do
      if (c >= 1 && group_any(!epilogue(c - 1), warp & 3)) {
        ok_all = false;
        break;
      }
    }
    // copies still in flight land before the CTA may exit
    if (AO_TMA) {
      if (ao_issuer && ao_pending >= 0) {
        const long long t0 = clock64();
        while (!mbar_test(aofull, (uint32_t)ao_pending) && clock64() - t0 < WAIT_BUDGET) {
        }
      }
    } else {
      asm volatile("cp.async.wait_all;" ::: "memory");
    }
    const bool last_ok = ok_all && epilogue(nks - 1);
    ok_all = !conv_any(!last_ok);  // every converter thread reaches this vote
    if (ok_all) {
      const double *stg = reinterpret_cast<const double *>(stages);
      for (int idx = threadIdx.x; idx < P.nocc * AH_TA * AH_TM; idx += 32 * AH_CONV) {
        const int ml = idx & 7, al = (idx >> 3) & 15, n = idx >> 7;
        const int ga = alpha0 + al, gm = mu0 + ml;
        if (ga < P.NBA && gm < P.nbas)
          P.half[((long long)n * P.NBA + ga) * P.nbas + gm] = stg[n * AH_STG + al * 9 + ml];
      }
    }
    if (threadIdx.x == 0 && armed >= 0 && *abort_flag) {
      // the last B copy completes before the CTA may exit
      const long long t0 = clock64();
      while (!mbar_test(sfull0 + 8 * armed_b, (uint32_t)armed) && clock64() - t0 < WAIT_BUDGET) {
      }
    }
  } else if (warp == AH_CONV) {
    // ------------------------------ MMA issuer -------------------------------
    if (lane == 0) {
      for (int c = 0; c < nks; ++c) {
        const int b = c & 1;
        if (!mbar_wait(sfull0 + 8 * b, (uint32_t)((c >> 1) & 1), abort_flag, P.err, 23)) break;
        if (c >= 2 &&
            !mbar_wait(aempty0 + 8 * b, (uint32_t)(((c - 2) >> 1) & 1), abort_flag, P.err, 24))
          break;
        tc_fence_after();
        const uint32_t sA = smem_u32(stages + b * STAGE);
        const uint32_t sB = sA + 3 * PANEL_BYTES;
        const uint32_t dL0 = tmem + (uint32_t)(b * 2 * NT);
        const uint32_t dL1 = dL0 + (uint32_t)NT;
#pragma unroll
        for (int k16 = 0; k16 < KSTEP / 16; ++k16) {
          const uint32_t koff = k16 * 32;
          const uint64_t a0 = smem_desc(sA + koff), a1 = smem_desc(sA + PANEL_BYTES + koff);
          const uint64_t a2 = smem_desc(sA + 2 * PANEL_BYTES + koff);
          const uint64_t b0 = smem_desc(sB + koff), b1 = smem_desc(sB + BPL + koff);
          const uint64_t b2 = smem_desc(sB + 2 * BPL + koff);
          const uint32_t acc = k16 > 0 ? 1u : 0u;  // each chunk starts its own sums
          mma_f16_id(dL0, a0, b0, P.idesc, acc);
          mma_f16_id(dL1, a0, b1, P.idesc, acc);
          mma_f16_id(dL1, a1, b0, P.idesc, 1u);
          mma_f16_id(dL1, a1, b1, P.idesc, 1u);
          mma_f16_id(dL1, a0, b2, P.idesc, 1u);
          mma_f16_id(dL1, a2, b0, P.idesc, 1u);
        }
        mma_commit(sempty0 + 8 * b);  // the stage may be refilled
        mma_commit(afull0 + 8 * b);   // the chunk's products are in TMEM
      }
      mma_commit(drain);
      const long long t0 = clock64();
      while (!mbar_test(drain, 0) && clock64() - t0 < WAIT_BUDGET) {
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == AH_CONV) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

// Occupied MO block sliced for ao_half_kernel: column n (orbital), chunk c of
// 64 nu values, scale per (column, chunk) with |x 2^e| <= 511.5; planes S0,
// R1, R2 at Bsl[(3 c + p) NT + n][64] (plain rows; the TMA copy swizzles
// them), scale 2^-e at sb[c NT + n].  One warp per (column, chunk); columns
// n >= nocc and nu >= nbas are zero.
__global__ void ao_occ_slice_kernel(const double *__restrict__ Cmo, int nbas, int nocc, int NT,
                                    int nks, __half *__restrict__ Bsl, float *__restrict__ sb) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= NT * nks) return;
  const int n = w % NT, c = w / NT;
  double v[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int nu = c * KSTEP + lane + 32 * q;
    v[q] = (n < nocc && nu < nbas) ? Cmo[(size_t)n * nbas + nu] : 0.0;
  }
  uint32_t key = 0;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const uint32_t kq =
        (uint32_t)(((unsigned long long)__double_as_longlong(v[q]) >> 32) & 0x7FFFFFFFu);
    key = kq > key ? kq : key;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint32_t other = __shfl_xor_sync(0xffffffffu, key, o);
    key = other > key ? other : key;
  }
  const int e = chunk_exponent_511(key);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    float qv, rv;
    split_int((unsigned long long)__double_as_longlong(v[q]), e, qv, rv);
    const __half h1 = __float2half_rn(rv);
    const size_t k = lane + 32 * q;
    Bsl[((size_t)(3 * c + 0) * NT + n) * 64 + k] = __float2half_rn(qv);
    Bsl[((size_t)(3 * c + 1) * NT + n) * 64 + k] = h1;
    Bsl[((size_t)(3 * c + 2) * NT + n) * 64 + k] = __float2half_rn(rv - __half2float(h1));
  }
  if (lane == 0) sb[(size_t)c * NT + n] = ldexpf(1.0f, -e);
}

// AO tensor rows: row m' = mu + nbas*alpha of (alpha|mu nu) over K = nu.
// One CTA owns 32 alpha x 8 mu rows, one thread per row, warps alpha-fastest
// so every load of a nu-step is one 256-byte segment.  Same scale rule and
// slice layout as slice_batch_kernel.  The FP16 slices of each 64-wide nu
// chunk are staged in shared memory (16-byte chunks XOR-swizzled by alpha)
// and written out row-contiguous: the 8 mu rows of one alpha are 1 KB of
// consecutive memory.  The first CTA also sets the scale of the padding rows
// (their slices are zeroed by the host).
constexpr int AO_TA = 32, AO_TM = 8, AO_ROWS = AO_TA * AO_TM;

__global__ void __launch_bounds__(AO_ROWS) ao_slice_kernel(const double *__restrict__ ao, int NBA,
                                                          int nbas, long long nrows_pad, int nks,
                                                          int nsl, long long plane,
                                                          __half *__restrict__ slices,
                                                          float *__restrict__ inv_scale) {
  extern __shared__ uint4 stage[];  // [nsl][AO_ROWS rows][8 chunks of 8 halves]
  const int a_l = threadIdx.x & (AO_TA - 1), m_l = threadIdx.x / AO_TA;
  const int al = blockIdx.x * AO_TA + a_l, mu = blockIdx.y * AO_TM + m_l;
  const bool live = (al < NBA) && (mu < nbas);
  const long long MK = (long long)NBA * nbas;
  const size_t kstride = (size_t)nrows_pad * 64;
  if (blockIdx.x == 0 && blockIdx.y == 0)
    for (long long t = MK + threadIdx.x; t < nrows_pad; t += blockDim.x) inv_scale[t] = 1.0f;
  // row (alpha, mu) over K = nu read along the middle index: (alpha|mu nu) =
  // (alpha|nu mu), 8 NBA bytes apart, so a row's values stay within a few
  // memory pages (along the last index they are 8 NBA nbas bytes apart)
  const double *src = ao + (live ? al + (size_t)MK * mu : 0);  // element nu at src[NBA*nu]
  int e = 0;
  if (live) {
    unsigned long long mxb = 0;
    float ss = 0.0f;
    // sixteen independent loads in flight per thread (one 256-byte segment
    // per warp each): the loop is bound by memory latency, not arithmetic
    for (int nu0 = 0; nu0 < nbas; nu0 += 16) {
      double v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = (nu0 + q < nbas) ? src[(size_t)NBA * (nu0 + q)] : 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const unsigned long long mag =
            (unsigned long long)__double_as_longlong(v[q]) & 0x7FFFFFFFFFFFFFFFull;
        mxb = mag > mxb ? mag : mxb;
        const float f = abs_trunc_f32(mag);
        ss = fmaf(f, f, ss);
      }
    }
    e = col_scale_exponent(mxb, ss, nbas);
  }
  const int rl = m_l + AO_TM * a_l;  // row within the CTA: the 8 mu of one alpha adjacent
  const int sw = a_l & 7;
  const __half hz = __float2half_rn(0.0f);
  for (int attempt = 0; attempt < 64; ++attempt) {
    long long n2 = 0;
    for (int kc = 0; kc < nks; ++kc) {
      for (int q00 = 0; q00 < 64; q00 += 16) {
        double v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int nu = kc * 64 + q00 + q;
          v[q] = (live && nu < nbas) ? src[(size_t)NBA * nu] : 0.0;
        }
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          __align__(16) __half h0[8], h1[8], h2[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int nu = kc * 64 + q00 + 8 * hh + q;
            h0[q] = h1[q] = h2[q] = hz;
            if (live && nu < nbas) {
              float qv, r;
              split_f32(v[8 * hh + q], e, qv, r);  // |x 2^e| <= 2047.5
              h0[q] = __float2half_rn(qv);
              h1[q] = __float2half_rn(r);
              h2[q] = __float2half_rn(r - __half2float(h1[q]));
              const int qi = __float_as_int(fabsf(qv) + 8388608.0f) - 0x4B000000;
              n2 += qi * qi;
            }
          }
          const int c = ((q00 >> 3) + hh) ^ sw;
          stage[(0 * AO_ROWS + rl) * 8 + c] = *reinterpret_cast<const uint4 *>(h0);
          if (nsl > 1) stage[(1 * AO_ROWS + rl) * 8 + c] = *reinterpret_cast<const uint4 *>(h1);
          if (nsl > 2) stage[(2 * AO_ROWS + rl) * 8 + c] = *reinterpret_cast<const uint4 *>(h2);
        }
      }
      __syncthreads();
      for (int j = threadIdx.x; j < AO_ROWS * 8; j += AO_ROWS) {
        const int r = j >> 3, c = j & 7;
        const int ra = r / AO_TM, rm = r % AO_TM;
        const int gal = blockIdx.x * AO_TA + ra, gmu = blockIdx.y * AO_TM + rm;
        if (gal < NBA && gmu < nbas) {
          const size_t row = (size_t)gmu + (size_t)nbas * gal;
          __half *dst = slices + (size_t)kc * kstride + row * 64 + c * 8;
          const int sc = c ^ (ra & 7);
          for (int sl = 0; sl < nsl; ++sl)
            *reinterpret_cast<uint4 *>(dst + sl * plane) = stage[(sl * AO_ROWS + r) * 8 + sc];
        }
      }
      __syncthreads();
    }
    // the norm bound makes a retry rare; the whole CTA repeats the pass with
    // a smaller scale on the rows that exceeded it
    const bool over = n2 > 16777216LL;
    if (!__syncthreads_or(over)) break;
    if (over) --e;
  }
  if (live) inv_scale[(size_t)mu + (size_t)nbas * al] = ldexpf(1.0f, -e);
}

}  // namespace

// A planned batch: up to three launch groups, workspace and (optionally)
// an instantiated CUDA graph of the whole evaluation.
struct SplitPlan {
  Group g[3];  // one residual slice (one-CTA), two residual slices, one residual slice (paired)
  PlainPlan *plain = nullptr;  // fragments planned in plain FP64 (slice count 0)
  int nsm = 0;
  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t graph = nullptr;
  // graph form of a plan with several launch groups: inputs on a side branch
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_in[3] = {nullptr, nullptr, nullptr};
  ~SplitPlan() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto &e : ev_in)
      if (e) cudaEventDestroy(e);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (side) cudaStreamDestroy(side);
    plain_plan_destroy(plain);
  }
  int launches() const {
    int n = plain_plan_launches(plain);
    for (auto &x : g)
      if (x.nfrag) n += 5;  // slicing, eps, kernel, two reductions
    return n;
  }
};

bool split_supported() { return get_encode() != nullptr; }

// Records the launch groups of a plan, one after the other (slicing, then
// the energy kernel and reductions of each group).  The overlapped form
// (RIMP2_BATCH_OVERLAP=1): with two or more groups, every group's inputs
// (slicing, orbital-energy pairs) go on a side branch, in the order the
// energy kernels run, and each energy kernel waits only for its own group's
// inputs, so the slicing of the next group runs while the current group's
// persistent kernel holds the SMs (a slicing block fits beside an energy
// CTA); the group with the least slicing work goes first, since nothing
// hides its inputs.
int record_plan_overlapped(SplitPlan *P, cudaStream_t s) {
  int order[3], n = 0;
  for (int k = 0; k < 3; ++k)
    if (P->g[k].nfrag) order[n++] = k;
  // measured on GB300 (256-fragment batch, same box, alternating runs):
  // 633.9 / 635.4 eff TFLOP/s with the groups one after the other against
  // 626.9 / 631.1 with the side branch -- under the power cap the slicing
  // beside an energy kernel costs that kernel more than it hides.  So the
  // groups run in sequence unless RIMP2_BATCH_OVERLAP=1.
  const char *ov = getenv("RIMP2_BATCH_OVERLAP");
  if (n < 2 || !(ov && ov[0] == '1')) {
    for (int k = 0; k < n; ++k) RIMP2_TRY(record_group(P->g[order[k]], s, P->nsm, nullptr));
    return RIMP2_OK;
  }
  int first = 0;
  for (int k = 1; k < n; ++k)
    if (P->g[order[k]].R < P->g[order[first]].R) first = k;  // R: 64-wide slice rows
  std::swap(order[0], order[first]);
  if (!P->side) {
    set_error("internal: side stream of the plan not created");
    return RIMP2_ERR_CUDA;
  }
  RIMP2_CK(cudaEventRecord(P->ev_fork, s));
  RIMP2_CK(cudaStreamWaitEvent(P->side, P->ev_fork, 0));
  for (int k = 0; k < n; ++k) {
    RIMP2_TRY(record_group_inputs(P->g[order[k]], P->side));
    RIMP2_CK(cudaEventRecord(P->ev_in[k], P->side));
  }
  for (int k = 0; k < n; ++k) {
    RIMP2_CK(cudaStreamWaitEvent(s, P->ev_in[k], 0));
    RIMP2_TRY(record_group(P->g[order[k]], s, P->nsm, nullptr, false));
  }
  return RIMP2_OK;
}

int split_plan_create(SplitPlan **out, int nfrag, const int *nocc, const int *nvirt, const int *NBA,
                      const double *const *Ca, const double *const *eo, const double *const *ev,
                      double *const *Epair, double *const *Etot, const int *nslices, bool graph,
                      cudaStream_t s) {
  *out = nullptr;
  // work items pack i | j << 16 and tA | tB << 16
  for (int f = 0; f < nfrag; ++f)
    if (nocc[f] > 65535 || (nvirt[f] + TILE - 1) / TILE > 65535) {
      set_error("split form: fragment %d too large for the work-item encoding (nocc=%d)", f,
                nocc[f]);
      return RIMP2_ERR_ARG;
    }
  SplitPlan *P = new SplitPlan();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&P->nsm, cudaDevAttrMultiProcessorCount, dev);
  P->g[0].nsl = 2;
  P->g[1].nsl = 3;
  P->g[2].nsl = 2;
  P->g[2].pair = true;
  std::vector<PlainFrag> plain;
  for (int f = 0; f < nfrag; ++f) {
    if (nslices && nslices[f] == 0) {
      PlainFrag F;
      memset(&F, 0, sizeof F);
      F.Ca = Ca[f];
      F.eo = eo[f];
      F.ev = ev[f];
      F.Epair = Epair[f];
      F.Etot = Etot[f];
      F.nocc = nocc[f];
      F.nvirt = nvirt[f];
      F.NBA = NBA[f];
      plain.push_back(F);
      continue;
    }
    FragDesc F;
    memset(&F, 0, sizeof F);
    F.nocc = nocc[f];
    F.nvirt = nvirt[f];
    F.NBA = NBA[f];
    F.Ca = Ca[f];
    F.eo = eo[f];
    F.ev = ev[f];
    F.Epair = Epair[f];
    F.Etot = Etot[f];
    const int ns = nslices ? nslices[f] : 1;
    P->g[ns >= 2 ? 1 : (pair_kernel_for(F.nocc, F.nvirt, F.NBA) ? 2 : 0)].fh.push_back(F);
  }
  for (auto &g : P->g) {
    if (g.fh.empty()) continue;
    int rc = build_group(g, s);
    if (rc != RIMP2_OK) {
      delete P;
      return rc;
    }
  }
  if (!plain.empty()) {
    int rc = plain_plan_create(&P->plain, (int)plain.size(), plain.data(), s);
    if (rc != RIMP2_OK) {
      delete P;
      return rc;
    }
  }
  if (graph) {
    int ngroups = 0;
    for (auto &g : P->g) ngroups += g.nfrag ? 1 : 0;
    if (ngroups >= 2) {  // the side branch of record_plan_overlapped
      if (cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&P->ev_in[0], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&P->ev_in[1], cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&P->ev_in[2], cudaEventDisableTiming) != cudaSuccess) {
        set_error("stream/event creation for the batch graph failed");
        delete P;
        return RIMP2_ERR_CUDA;
      }
    }
    // the captured sequence needs the workspace already in place
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      set_error("graph capture start failed: %s", cudaGetErrorString(e));
      delete P;
      return RIMP2_ERR_CUDA;
    }
    const long long n0 = rimp2_kernel_launch_count();
    int rc = plain_plan_record(P->plain, s);
    if (rc == RIMP2_OK) rc = record_plan_overlapped(P, s);
    e = cudaStreamEndCapture(s, &P->graph);
    // captured launches run at each graph launch, not here
    count_launch(-(int)(rimp2_kernel_launch_count() - n0));
    if (rc != RIMP2_OK || e != cudaSuccess) {
      if (rc == RIMP2_OK) set_error("graph capture failed: %s", cudaGetErrorString(e));
      delete P;
      return rc != RIMP2_OK ? rc : RIMP2_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&P->gexec, P->graph, 0);
    if (e != cudaSuccess) {
      set_error("graph instantiate failed: %s", cudaGetErrorString(e));
      delete P;
      return RIMP2_ERR_CUDA;
    }
  }
  *out = P;
  return RIMP2_OK;
}

int split_plan_execute(SplitPlan *P, cudaStream_t s) {
  if (P->gexec) {
    RIMP2_CK(cudaGraphLaunch(P->gexec, s));
    count_launch(P->launches());
    return RIMP2_OK;
  }
  const bool timed = timing_enabled();
  cudaEvent_t ev[4];
  if (timed)
    for (int k = 0; k < 4; ++k) RIMP2_CK(cudaEventCreate(&ev[k]));
  // a plan of plain fragments only is timed as one kernel interval
  const bool plain_only = !P->g[0].nfrag && !P->g[1].nfrag && !P->g[2].nfrag;
  if (timed && plain_only) {
    RIMP2_CK(cudaEventRecord(ev[0], s));
    RIMP2_CK(cudaEventRecord(ev[1], s));
  }
  RIMP2_TRY(plain_plan_record(P->plain, s));
  if (timed && plain_only) RIMP2_CK(cudaEventRecord(ev[2], s));
  for (auto &g : P->g) RIMP2_TRY(record_group(g, s, P->nsm, timed ? ev : nullptr));
  if (timed) {
    RIMP2_CK(cudaEventRecord(ev[3], s));
    RIMP2_CK(cudaEventSynchronize(ev[3]));
    float ms;
    for (int k = 0; k < 3; ++k) {
      RIMP2_CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
      record_timing(k, ms);
    }
    for (int k = 0; k < 4; ++k) cudaEventDestroy(ev[k]);
  }
  return RIMP2_OK;
}

void split_plan_destroy(SplitPlan *P) { delete P; }

// Execution of a plan (no graph) whose inputs are still in host memory:
// copy c moves count[c] doubles from src[c] to dst[c].  The copies run on the
// copy streams cs[0..ncs) launch group by launch group, the group with the
// least Calpha first; copies that belong to no split group (orbital
// energies, the plain FP64 fragments) go before all of them.  Within a
// group each copy goes to the stream with the fewest bytes so far (the
// batched host call passes one stream: four were measured slower).  Each
// group's slicing waits only
// for its own fragments' copies, so the transfer of the later, larger
// groups overlaps the kernels of the earlier ones.  A copy belongs to the
// group whose fragment has dst as its Calpha address.  Several plans over
// one set of buffers run in turn: the first call waits for the allocation
// (wait_alloc), the later ones queue their copies behind its copies.
int split_plan_execute_host(SplitPlan *P, cudaStream_t s, const cudaStream_t *cs, int ncs,
                            int ncopy, double *const *dst, const double *const *src,
                            const size_t *count, bool wait_alloc) {
  struct Events {
    std::vector<cudaEvent_t> e;
    ~Events() {
      for (auto x : e) cudaEventDestroy(x);
    }
  } ev;
  auto event = [&](cudaEvent_t *out) -> int {
    RIMP2_CK(cudaEventCreateWithFlags(out, cudaEventDisableTiming));
    ev.e.push_back(*out);
    return RIMP2_OK;
  };
  std::vector<int> owner(ncopy, -1);  // launch group of each copy, -1: none
  size_t bytes[3] = {0, 0, 0};
  int order[3], n = 0;
  for (int k = 0; k < 3; ++k) {
    for (const auto &F : P->g[k].fh) {
      bytes[k] += (size_t)F.NBA * F.nvirt * F.nocc;
      for (int c = 0; c < ncopy; ++c)
        if (dst[c] == F.Ca) owner[c] = k;
    }
    if (P->g[k].nfrag) order[n++] = k;
  }
  std::sort(order, order + n, [&](int a, int b) { return bytes[a] < bytes[b]; });
  // the copy streams start after the destination buffers' allocation on s
  // (wait_alloc false: an earlier call on these streams already waited)
  if (wait_alloc) {
    cudaEvent_t e0;
    RIMP2_TRY(event(&e0));
    RIMP2_CK(cudaEventRecord(e0, s));
    for (int q = 0; q < ncs; ++q) RIMP2_CK(cudaStreamWaitEvent(cs[q], e0, 0));
  }
  // phase 0: copies outside the split groups; phase 1 + k: group order[k]
  std::vector<cudaEvent_t> done((size_t)(1 + n) * ncs);
  for (int ph = 0; ph <= n; ++ph) {
    const int want = ph == 0 ? -1 : order[ph - 1];
    std::vector<size_t> load(ncs, 0);
    for (int c = 0; c < ncopy; ++c) {
      if (owner[c] != want) continue;
      const int q = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[q] += count[c];
      RIMP2_CK(cudaMemcpyAsync(dst[c], src[c], count[c] * sizeof(double), cudaMemcpyHostToDevice,
                               cs[q]));
    }
    for (int q = 0; q < ncs; ++q) {
      RIMP2_TRY(event(&done[(size_t)ph * ncs + q]));
      RIMP2_CK(cudaEventRecord(done[(size_t)ph * ncs + q], cs[q]));
    }
  }
  for (int q = 0; q < ncs; ++q) RIMP2_CK(cudaStreamWaitEvent(s, done[q], 0));
  RIMP2_TRY(plain_plan_record(P->plain, s));
  for (int k = 0; k < n; ++k) {
    for (int q = 0; q < ncs; ++q)
      RIMP2_CK(cudaStreamWaitEvent(s, done[(size_t)(1 + k) * ncs + q], 0));
    RIMP2_TRY(record_group(P->g[order[k]], s, P->nsm, nullptr));
  }
  return RIMP2_OK;
}

int bounded_wait_selftest(long long budget_cycles, cudaStream_t s) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(budget_cycles, device_error_word());
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return collect_device_error(s);
}

int rcp_denom_selftest(int n, const float *d, float *r, float *ref, cudaStream_t s) {
  DevBuf dd, dr, dref;
  const size_t b = sizeof(float) * (size_t)n;
  RIMP2_TRY(dd.alloc(b, s));
  RIMP2_TRY(dr.alloc(b, s));
  RIMP2_TRY(dref.alloc(b, s));
  RIMP2_CK(cudaMemcpyAsync(dd.p, d, b, cudaMemcpyHostToDevice, s));
  rcp_selftest_kernel<<<(n + 255) / 256, 256, 0, s>>>(dd.as<float>(), dr.as<float>(),
                                                      dref.as<float>(), n);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  RIMP2_CK(cudaMemcpyAsync(r, dr.p, b, cudaMemcpyDeviceToHost, s));
  RIMP2_CK(cudaMemcpyAsync(ref, dref.p, b, cudaMemcpyDeviceToHost, s));
  RIMP2_CK(cudaStreamSynchronize(s));
  return RIMP2_OK;
}

// Host Calpha -> energies with the copy overlapped: occupied indices are
// copied in chunks on a second stream; once chunk c has landed, its columns
// are sliced and the work items of every pair (i <= j) with j in chunk c --
// whose inputs are then all on the device -- run as one persistent launch,
// while chunk c+1 is still in flight.  dCa must have room for the fragment.
int split_energy_streamed(const double *hCa, double *dCa, const SplitEnergyArgs &a,
                          cudaStream_t s, cudaStream_t copy_s, int chunk_occ) {
  // Occupied-index chunk boundaries: the first chunk small (its copy is the
  // only one nothing hides), later ones growing by half, since chunk c's
  // work grows with its column indices j while its copy does not; chunk_occ
  // caps the first chunk.  Chunk c is sliced on the slicing stream as soon
  // as its copy lands, beside chunk c-1's energy kernel, and its energy
  // kernel starts once it is sliced, so after the first few chunks the copy
  // engine and the slicer run ahead of the tensor cores.
  std::vector<int> bnd;
  for (int b = std::min(a.nocc, std::max(1, std::min(chunk_occ, 4))); ;) {
    bnd.push_back(b);
    if (b >= a.nocc) break;
    b = std::min(a.nocc, b + std::max(1, b / 2));
  }
  if (inject_fault("launch")) {  // before any copy is in flight
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  SplitPlan *P = nullptr;
  const int ns = a.nslices;
  const double *dCaC = dCa;
  RIMP2_TRY(split_plan_create(&P, 1, &a.nocc, &a.nvirt, &a.NBA, &dCaC, &a.eo, &a.ev, &a.Epair,
                              &a.Etot, &ns, false, s));
  Group &g = P->g[0].nfrag ? P->g[0] : (P->g[1].nfrag ? P->g[1] : P->g[2]);
  const FragDesc &F = g.fh[0];
  const FragDesc *fr = g.frags.as<FragDesc>();
  int rc = RIMP2_OK;
  const int nchunk = (int)bnd.size();
  // ev[c]: chunk c copied (copy stream); ev[nchunk + c]: chunk c sliced
  // (slicing stream); ev[2 nchunk]: the plan's buffers exist (stream s)
  std::vector<cudaEvent_t> ev(2 * nchunk + 1, nullptr);
  for (auto &e : ev)
    if (rc == RIMP2_OK && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      set_error("event creation failed");
      rc = RIMP2_ERR_CUDA;
    }
  // RIMP2_STREAM_SLICE=0: slice on s, between the energy launches
  const char *sv = getenv("RIMP2_STREAM_SLICE");
  cudaStream_t ss = (sv && sv[0] == '0') ? s : slice_stream();
  if (rc == RIMP2_OK && !ss) {
    set_error("slicing stream unavailable");
    rc = RIMP2_ERR_CUDA;
  }
  const size_t slab = (size_t)a.NBA * a.nvirt;  // doubles per occupied index
  // copies first, so the copy engine runs ahead of the compute stream
  for (int c = 0; c < nchunk && rc == RIMP2_OK; ++c) {
    const int i0 = c ? bnd[c - 1] : 0, i1 = bnd[c];
    cudaError_t e = cudaMemcpyAsync(dCa + slab * i0, hCa + slab * i0, sizeof(double) * slab * (i1 - i0),
                                    cudaMemcpyHostToDevice, copy_s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[c], copy_s);
    if (e != cudaSuccess) {
      set_error("streamed copy failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
    }
  }
  if (rc == RIMP2_OK) {
    dim3 g2((unsigned)((g.max_nv + 255) / 256), 1);
    eps_batch_kernel<<<g2, 256, 0, s>>>(fr, g.eo2.as<float2>(), g.ev2.as<float2>());
    count_launch(1);
  }
  // slicing of every chunk on the slicing stream, each after its copy (and
  // after the plan's buffers, allocated on s); columns of different chunks
  // are disjoint in the slices, scales and corrections
  if (rc == RIMP2_OK) {
    cudaError_t e = cudaEventRecord(ev[2 * nchunk], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ss, ev[2 * nchunk], 0);
    for (int c = 0; c < nchunk && e == cudaSuccess; ++c) {
      const int i0 = c ? bnd[c - 1] : 0, i1 = bnd[c];
      const int col0 = i0 * F.nvpad, col1 = i1 * F.nvpad;
      e = cudaStreamWaitEvent(ss, ev[c], 0);
      if (e != cudaSuccess) break;
      slice_batch_kernel<<<(unsigned)(((long long)(col1 - col0) * 32 + 255) / 256), 256, 0, ss>>>(
          fr, g.nsl, g.R * 64, g.slices.as<__half>(), g.inv.as<float>(), col0, col1,
          g.pair ? 1 : 0, g.dcorr.as<float>());
      count_launch(1);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(ev[nchunk + c], ss);
    }
    if (e != cudaSuccess) {
      set_error("streamed slicing failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
    }
  }
  BatchParams BP;
  BP.frags = fr;
  BP.items = g.items.as<int4>();
  BP.eo2 = g.eo2.as<float2>();
  BP.ev2 = g.ev2.as<float2>();
  BP.inv_scale = g.inv.as<float>();
  BP.part = g.part.as<double>();
  BP.err = device_error_word();
  for (int c = 0; c < nchunk && rc == RIMP2_OK; ++c) {
    const int i0 = c ? bnd[c - 1] : 0, i1 = bnd[c];
    cudaError_t e = cudaStreamWaitEvent(s, ev[nchunk + c], 0);
    if (e != cudaSuccess) {
      set_error("stream wait failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
      break;
    }
    e = cudaMemsetAsync(g.queue.p, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) {
      set_error("queue reset failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
      break;
    }
    if (g.pair) {
      // pair items with j in [i0, i1) (their i0' < i0'+1 <= j are already copied)
      PairParams Q;
      Q.frags = fr;
      Q.items = g.pitems.as<int4>();
      Q.item_begin = pair_items_before(i0) * F.ntp;
      Q.nitems = pair_items_before(i1) * F.ntp;
      Q.dcorr = g.dcorr.as<float>();
      Q.queue = g.queue.as<unsigned int>();
      Q.eo2 = BP.eo2;
      Q.ev2 = BP.ev2;
      Q.inv_scale = BP.inv_scale;
      Q.part = BP.part;
      Q.err = BP.err;
      const int npair = (int)std::min<long long>(Q.nitems - Q.item_begin, std::max(1, P->nsm / 2));
      note_split_kernel(2);
      rc = launch_pair(g, Q, npair, s);
      if (rc != RIMP2_OK) break;
    } else {
      // pairs (i<=j) with j in [i0, i1): pair indices [i0(i0+1)/2, i1(i1+1)/2)
      const long long pb = (long long)i0 * (i0 + 1) / 2, pe = (long long)i1 * (i1 + 1) / 2;
      BP.item_begin = pb * F.ntp;
      BP.nitems = pe * F.ntp;
      BP.queue = g.queue.as<unsigned int>();
      const int grid = (int)std::min<long long>(BP.nitems - BP.item_begin, P->nsm);
      note_split_kernel(1);
      // at the highest priority, like the paired kernel: the next chunk's
      // slicing blocks wait behind this kernel's CTAs, not ahead of them
      if (g.nsl == 2)
        e = launch_hi(split_batch_kernel<2, 3>, grid, BATCH_THREADS, smem_bytes(2, 3), s, g.tm, BP);
      else
        e = launch_hi(split_batch_kernel<3, 2>, grid, BATCH_THREADS, smem_bytes(3, 2), s, g.tm, BP);
      if (e != cudaSuccess) {
        set_error("split launch failed: %s", cudaGetErrorString(e));
        rc = RIMP2_ERR_CUDA;
        break;
      }
    }
    count_launch(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("split launch failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
    }
  }
  if (rc == RIMP2_OK) {
    pair_reduce_batch_kernel<<<(unsigned)((g.npairs_total + 7) / 8), 256, 0, s>>>(
        fr, g.nfrag, g.npairs_total, g.part.as<double>());
    total_reduce_batch_kernel<<<g.nfrag, 1024, 0, s>>>(fr);
    count_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("reduction launch failed: %s", cudaGetErrorString(e));
      rc = RIMP2_ERR_CUDA;
    }
  }
  // on failure, copies may still be in flight into dCa: finish them before
  // the caller can release dCa
  if (rc != RIMP2_OK) {
    cudaStreamSynchronize(copy_s);
    if (ss && ss != s) cudaStreamSynchronize(ss);
    cudaStreamSynchronize(s);
  }
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  split_plan_destroy(P);
  return rc;
}

// ---- general split GEMM: host side -------------------------------------------
int sliced_cols(SlicedOp &op, const double *src, int K, int nrows, int ngroups, int nsl,
                cudaStream_t s) {
  FragDesc F;
  memset(&F, 0, sizeof F);
  F.nocc = ngroups;
  F.nvirt = nrows;
  F.NBA = K;
  F.nvpad = (nrows + TILE - 1) / TILE * TILE;
  F.nks = (K + KSTEP - 1) / KSTEP;
  F.ncol = ngroups * F.nvpad;
  F.Ca = src;
  op.nsl = nsl;
  op.nks = F.nks;
  op.rows_per_group = F.nvpad;
  op.ncol = F.ncol;
  op.R = (long long)F.nks * F.ncol;
  if (op.R > 2147483647LL - TILE) {
    set_error("split GEMM operand too large (%lld rows)", op.R);
    return RIMP2_ERR_ARG;
  }
  RIMP2_TRY(op.desc.alloc(sizeof(FragDesc), s));
  RIMP2_CK(cudaMemcpyAsync(op.desc.p, &F, sizeof F, cudaMemcpyHostToDevice, s));
  RIMP2_TRY(op.slices.alloc(sizeof(__half) * (size_t)nsl * op.R * 64, s));
  RIMP2_TRY(op.inv.alloc(sizeof(float) * (size_t)op.ncol, s));
  slice_batch_kernel<<<(unsigned)(((long long)F.ncol * 32 + 255) / 256), 256, 0, s>>>(
      op.desc.as<FragDesc>(), nsl, op.R * 64, op.slices.as<__half>(), op.inv.as<float>(), 0,
      0x7fffffff);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

int sliced_ao(SlicedOp &op, const double *ao, int NBA, int nbas, int nsl, cudaStream_t s) {
  const long long rows = (long long)NBA * nbas;
  op.nsl = nsl;
  op.nks = (nbas + KSTEP - 1) / KSTEP;
  op.ncol = (rows + TILE - 1) / TILE * TILE;
  op.rows_per_group = op.ncol;
  op.R = (long long)op.nks * op.ncol;
  if (op.R > 2147483647LL - TILE) {
    set_error("AO operand too large (%lld rows)", op.R);
    return RIMP2_ERR_ARG;
  }
  RIMP2_TRY(op.slices.alloc(sizeof(__half) * (size_t)nsl * op.R * 64, s));
  RIMP2_TRY(op.inv.alloc(sizeof(float) * (size_t)op.ncol, s));
  // padding rows [rows, ncol) of every K chunk of every slice plane: the
  // chunks are equally spaced (ncol rows of 128 bytes) across the planes
  if (op.ncol > rows)
    RIMP2_CK(cudaMemset2DAsync(op.slices.as<__half>() + (size_t)rows * 64, (size_t)op.ncol * 128,
                               0, (size_t)(op.ncol - rows) * 128, (size_t)op.nks * nsl, s));
  const int smem = nsl * AO_ROWS * 128;
  RIMP2_CK(cudaFuncSetAttribute(ao_slice_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  dim3 grid((unsigned)((NBA + AO_TA - 1) / AO_TA), (unsigned)((nbas + AO_TM - 1) / AO_TM));
  ao_slice_kernel<<<grid, AO_ROWS, smem, s>>>(ao, NBA, nbas, op.ncol, op.nks, nsl, op.R * 64,
                                              op.slices.as<__half>(), op.inv.as<float>());
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

static int encode_op(CUtensorMap &tm, const SlicedOp &op, int boxrows) {
  auto encode = get_encode();
  if (!encode) {
    set_error("cuTensorMapEncodeTiled entry point unavailable");
    return RIMP2_ERR_UNSUPPORTED;
  }
  cuuint64_t dims[3] = {64, (cuuint64_t)op.R, (cuuint64_t)op.nsl};
  cuuint64_t strides[2] = {128, (cuuint64_t)op.R * 128};
  cuuint32_t box[3] = {KSTEP, (cuuint32_t)boxrows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult cr = encode(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, op.slices.p, dims, strides, box,
                       estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return RIMP2_ERR_CUDA;
  }
  return RIMP2_OK;
}

int split_gemm(const SlicedOp &A, long long a_row0, long long a_bstride, const SlicedOp &B,
               long long b_row0, long long b_bstride, int M, int N, int nbatch, double *out,
               long long sOm, long long sOn, long long sOb, cudaStream_t s) {
  if (A.nsl != B.nsl || A.nks != B.nks || M <= 0 || N <= 0 || nbatch <= 0) {
    set_error("split_gemm: operand mismatch or bad sizes");
    return RIMP2_ERR_ARG;
  }
  GemmSP P;
  memset(&P, 0, sizeof P);
  P.M = M;
  P.N = N;
  P.NT = N <= TILE ? (N + 15) / 16 * 16 : TILE;
  P.nks = A.nks;
  P.mtiles = (M + TILE - 1) / TILE;
  P.ntiles = (N + P.NT - 1) / P.NT;
  P.nbatch = nbatch;
  P.a_ncol = A.ncol;
  P.b_ncol = B.ncol;
  P.a_row0 = a_row0;
  P.a_bstride = a_bstride;
  P.b_row0 = b_row0;
  P.b_bstride = b_bstride;
  P.a_inv = A.inv.as<float>();
  P.b_inv = B.inv.as<float>();
  P.out = out;
  P.sOm = sOm;
  P.sOn = sOn;
  P.sOb = sOb;
  uint32_t cols = 32;
  while (cols < (uint32_t)(4 * P.NT)) cols <<= 1;
  P.tmem_cols = cols;
  P.err = device_error_word();
  const long long nitems = (long long)nbatch * P.mtiles * P.ntiles;
  if (nitems > 2147483647LL) {
    set_error("split_gemm: too many tiles");
    return RIMP2_ERR_ARG;
  }
  CUtensorMap tA, tB;
  RIMP2_TRY(encode_op(tA, A, TILE));
  RIMP2_TRY(encode_op(tB, B, P.NT));
  const int smem = gemm_smem_bytes(A.nsl, P.NT);
  auto kern = A.nsl == 3 ? split_gemm_kernel<3> : split_gemm_kernel<2>;
  RIMP2_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int dev = 0, nsm = 0, resident = 0;
  RIMP2_CK(cudaGetDevice(&dev));
  RIMP2_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  RIMP2_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, GEMM_THREADS, smem));
  // persistent CTAs whose TMEM allocations fit an SM together
  resident = std::max(1, std::min(resident, (int)(512 / cols)));
  const long long grid = std::min<long long>(nitems, (long long)nsm * resident);
  kern<<<(unsigned)grid, GEMM_THREADS, smem, s>>>(tA, tB, P);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

// First half of the AO->MO transform, fused (ao_half_kernel): the occupied MO
// block is sliced per (column, 64-wide nu chunk), then one pass over the AO
// tensor forms half[i][alpha][mu].  *handled = false (nothing launched) when
// nocc exceeds the kernel's 80 columns; the caller then takes the sliced path.
int ao_half_fused(const double *ao, int NBA, int nbas, const double *Cmo, int nocc, double *half,
                  cudaStream_t s, bool *handled) {
  *handled = false;
  const int NT = (nocc + 15) / 16 * 16;
  if (NT > AH_NT_MAX || nocc <= 0) return RIMP2_OK;
  const char *env = getenv("RIMP2_AO_FUSED");  // =0: the sliced first half (for comparisons)
  if (env && env[0] == '0') return RIMP2_OK;
  auto encode = get_encode();
  if (!encode) {
    set_error("cuTensorMapEncodeTiled entry point unavailable");
    return RIMP2_ERR_UNSUPPORTED;
  }
  const int nks = (nbas + KSTEP - 1) / KSTEP;
  const long long ntiles = (long long)((NBA + AH_TA - 1) / AH_TA) * ((nbas + AH_TM - 1) / AH_TM);
  if (ntiles > 2147483647LL) {
    set_error("AO transform too large for one launch (%lld tiles)", ntiles);
    return RIMP2_ERR_ARG;
  }
  DevBuf Bsl, sb;
  RIMP2_TRY(Bsl.alloc(sizeof(__half) * (size_t)3 * nks * NT * 64, s));
  RIMP2_TRY(sb.alloc(sizeof(float) * (size_t)nks * NT, s));
  const long long nw = (long long)NT * nks;
  ao_occ_slice_kernel<<<(unsigned)((nw * 32 + 255) / 256), 256, 0, s>>>(
      Cmo, nbas, nocc, NT, nks, Bsl.as<__half>(), sb.as<float>());
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  CUtensorMap tm;
  cuuint64_t dims[3] = {64, (cuuint64_t)NT, (cuuint64_t)(3 * nks)};
  cuuint64_t strides[2] = {128, (cuuint64_t)NT * 128};
  cuuint32_t box[3] = {KSTEP, (cuuint32_t)NT, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult cr = encode(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, Bsl.p, dims, strides, box, estr,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return RIMP2_ERR_CUDA;
  }
  AoHalfParams P;
  P.ao = ao;
  P.NBA = NBA;
  P.nbas = nbas;
  P.nocc = nocc;
  P.NT = NT;
  P.nks = nks;
  P.ta_tiles = (NBA + AH_TA - 1) / AH_TA;
  P.sb = sb.as<float>();
  P.half = half;
  P.idesc = (1u << 4) | ((uint32_t)(NT >> 3) << 17) | ((uint32_t)(TILE >> 4) << 24);
  P.err = device_error_word();
  // The AO chunks arrive by TMA (one 16 alpha x 64 nu x 2 mu box per row
  // group) when the tensor's strides allow it (NBA even: 16-byte multiples)
  // and its base is 16-byte aligned; otherwise by per-thread cp.async.
  CUtensorMap tmAO;
  memset(&tmAO, 0, sizeof tmAO);
  const bool ao_tma = (NBA % 2 == 0) && ((uintptr_t)ao % 16 == 0);
  if (ao_tma) {
    cuuint64_t adims[3] = {(cuuint64_t)NBA, (cuuint64_t)nbas, (cuuint64_t)nbas};
    cuuint64_t astr[2] = {(cuuint64_t)NBA * 8, (cuuint64_t)NBA * nbas * 8};
    cuuint32_t abox[3] = {AH_TA, KSTEP, 2};
    cr = encode(&tmAO, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double *>(ao), adims, astr,
                abox, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) {
      set_error("cuTensorMapEncodeTiled (AO tensor) failed (%d)", (int)cr);
      return RIMP2_ERR_CUDA;
    }
  }
  auto kern = ao_tma ? ao_half_kernel<true> : ao_half_kernel<false>;
  const int smem = ah_smem_bytes(NT);
  RIMP2_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int resident = 0;
  RIMP2_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, kern, AH_THREADS, smem));
  if (resident < 1) return RIMP2_OK;  // cannot be resident here: the sliced path runs
  kern<<<(unsigned)ntiles, AH_THREADS, smem, s>>>(tm, tmAO, P);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  *handled = true;
  return RIMP2_OK;
}

// Local-orbital fragment energy in the split form: slices of Calpha and of its
// projected copy Ct in one buffer, one persistent split_eos_kernel launch,
// compensated FP64 pair and total reductions.
int split_eos_energy(const double *Ca, const double *Ct, int NBA, int nvirt, int nocc,
                     const double *eo, const double *ev, double *Epair, double *Etot,
                     int nslices, cudaStream_t s) {
  const int nsl = nslices + 1;
  auto encode = get_encode();
  if (!encode) {
    set_error("cuTensorMapEncodeTiled entry point unavailable");
    return RIMP2_ERR_UNSUPPORTED;
  }
  FragDesc fh[2];
  memset(fh, 0, sizeof fh);
  const int nvpad = (nvirt + TILE - 1) / TILE * TILE;
  const int nks = (NBA + KSTEP - 1) / KSTEP;
  const int nt = nvpad / TILE;
  const int ntp = nt * (nt + 1) / 2;
  const long long ncol = (long long)nocc * nvpad;
  const long long R = 2LL * nks * ncol;
  const int npairs = nocc * (nocc + 1) / 2;
  const long long nitems = (long long)npairs * ntp * 2;
  if (R > 2147483647LL - TILE || nitems > 2147483647LL || ncol > 2147483647LL) {
    set_error("split local-orbital energy: fragment too large (rows=%lld, items=%lld)", R, nitems);
    return RIMP2_ERR_ARG;
  }
  for (int f = 0; f < 2; ++f) {
    FragDesc &F = fh[f];
    F.nocc = nocc;
    F.nvirt = nvirt;
    F.nvpad = nvpad;
    F.NBA = NBA;
    F.nks = nks;
    F.ntp = ntp;
    F.ncol = (int)ncol;
    F.row_base = (long long)f * nks * ncol;
    F.col_base = (long long)f * ncol;
    F.Ca = f ? Ct : Ca;
    F.eo = eo;
    F.ev = ev;
  }
  const int vplane = nsl == 2 ? 1 : 0;  // one residual slice: V plane, three products
  const int planes = nsl + vplane;
  DevBuf frags, slices, inv, eo2, ev2, part, queue, pairs, dcorr;
  RIMP2_TRY(frags.alloc(sizeof fh, s));
  RIMP2_TRY(slices.alloc(sizeof(__half) * (size_t)planes * R * 64, s));
  RIMP2_TRY(inv.alloc(sizeof(float) * 2 * (size_t)ncol, s));
  if (vplane) RIMP2_TRY(dcorr.alloc(sizeof(float) * 2 * (size_t)ncol, s));
  RIMP2_TRY(eo2.alloc(sizeof(float2) * nocc, s));
  RIMP2_TRY(ev2.alloc(sizeof(float2) * nvpad, s));
  RIMP2_TRY(part.alloc(sizeof(double) * (size_t)nitems, s));
  RIMP2_TRY(queue.alloc(sizeof(unsigned int), s));
  RIMP2_TRY(pairs.alloc(sizeof(int) * 2 * (size_t)npairs, s));
  RIMP2_CK(cudaMemcpyAsync(frags.p, fh, sizeof fh, cudaMemcpyHostToDevice, s));
  const FragDesc *fr = frags.as<FragDesc>();
  slice_batch_kernel<<<dim3((unsigned)((ncol * 32 + 255) / 256), 2), 256, 0, s>>>(
      fr, nsl, R * 64, slices.as<__half>(), inv.as<float>(), 0, 0x7fffffff, vplane,
      dcorr.as<float>());
  eps_batch_kernel<<<dim3((unsigned)((std::max(nvpad, nocc) + 255) / 256), 1), 256, 0, s>>>(
      fr, eo2.as<float2>(), ev2.as<float2>());
  count_launch(2);
  CUtensorMap tmA, tmB;
  cuuint64_t dims[3] = {64, (cuuint64_t)R, (cuuint64_t)planes};
  cuuint64_t strides[2] = {128, (cuuint64_t)R * 128};
  cuuint32_t boxA[3] = {KSTEP, TILE, 1}, boxB[3] = {KSTEP, HALF, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult cr = encode(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, slices.p, dims, strides, boxA,
                       estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr == CUDA_SUCCESS)
    cr = encode(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, slices.p, dims, strides, boxB, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)cr);
    return RIMP2_ERR_CUDA;
  }
  EosParams P;
  P.inv = inv.as<float>();
  P.eo2 = eo2.as<float2>();
  P.ev2 = ev2.as<float2>();
  P.nitems = nitems;
  P.queue = queue.as<unsigned int>();
  P.part = part.as<double>();
  P.err = device_error_word();
  P.nocc = nocc;
  P.nvirt = nvirt;
  P.nvpad = nvpad;
  P.nks = nks;
  P.ntp = ntp;
  P.ncol = (int)ncol;
  P.rowC = 0;
  P.rowCt = (int)((long long)nks * ncol);
  P.dcorr = dcorr.as<float>();
  int dev = 0, nsm = 0;
  RIMP2_CK(cudaGetDevice(&dev));
  RIMP2_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = (int)std::min<long long>(nitems, nsm);
  RIMP2_CK(cudaMemsetAsync(queue.p, 0, sizeof(unsigned int), s));
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  if (nsl == 2) {
    RIMP2_CK(cudaFuncSetAttribute(split_eos_kernel<2, 4>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, eos_smem_bytes(2, 4)));
    split_eos_kernel<2, 4><<<grid, NTHREADS, eos_smem_bytes(2, 4), s>>>(tmA, tmB, P);
  } else {
    RIMP2_CK(cudaFuncSetAttribute(split_eos_kernel<3, 3>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, eos_smem_bytes(3, 3)));
    split_eos_kernel<3, 3><<<grid, NTHREADS, eos_smem_bytes(3, 3), s>>>(tmA, tmB, P);
  }
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  make_pairs_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(nocc, pairs.as<int>());
  RIMP2_CK(cudaMemsetAsync(Epair, 0, sizeof(double) * (size_t)nocc * nocc, s));
  pair_reduce_kernel<<<(npairs + 7) / 8, 256, 0, s>>>(part.as<double>(), 2 * ntp, pairs.as<int>(),
                                                     npairs, nocc, Epair);
  total_reduce_kernel<<<1, 1024, 0, s>>>(Epair, nocc, Etot);
  count_launch(3);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

int split_energy(const SplitEnergyArgs &a, cudaStream_t s, float *ms_kernel) {
  (void)ms_kernel;
  SplitPlan *P = nullptr;
  const int ns = a.nslices;
  RIMP2_TRY(split_plan_create(&P, 1, &a.nocc, &a.nvirt, &a.NBA, &a.Ca, &a.eo, &a.ev, &a.Epair,
                              &a.Etot, &ns, false, s));
  int rc = split_plan_execute(P, s);
  split_plan_destroy(P);  // workspace is released stream-ordered
  return rc;
}

}  // namespace rimp2
