// front_end.cu -- Calpha from AO three-centre integrals on the GPU.
//
//   (alpha|a i) = sum_{mu,nu} Cmo(mu,nocc+a) Cmo(nu,i) (alpha|mu nu)
//   V = L L^T (Cholesky of the auxiliary metric)
//   Calpha(:,a,i) = L^{-1} (:|a i)
// so that sum_alpha Calpha(alpha,a,i) Calpha(alpha,b,j) = (ai|V^{-1}|bj).
// The reference starts from Calpha (RIMP2.F90:48-49); this front end has no
// counterpart there.  The AO->MO transform runs either on the FP64 DMMA GEMM
// of fp64_kernels.cu or on the tcgen05 split GEMM (two residual FP16 slices,
// ~2^-33 relative per product); the Cholesky and the solve are FP64, blocked
// (64) so that all but O(n*64^2) of their work is GEMM:
//   Cholesky: diagonal-block factorisation and inverse (one CTA), panel
//             P L_kk^{-T} (GEMM), trailing update C -= P P^T on the
//             lower-triangle tiles;
//   solve:    all diagonal-block inverses in one launch, then
//             X_k = inv(L_kk) B_k and B_rest -= L_rest,k X_k (GEMMs).
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace rimp2 {
void count_launch(int n);

namespace {

constexpr int NB = 64;

GemmDesc gdesc() {
  GemmDesc g;
  memset(&g, 0, sizeof g);
  g.alpha = 1.0;
  g.beta = 0.0;
  g.nb0 = g.nb1 = 1;
  return g;
}

// Diagonal 64x64 blocks: factorisation and triangular inverse in shared
// memory, 256 threads.  Blocks narrower than 64 (the last one) are padded
// with the identity, so the same code runs on every block.
constexpr int DP = NB + 1;                        // padded row (doubles)
constexpr int DIAG_SMEM = (2 * NB * DP + 5 * NB + 1) * sizeof(double);

__device__ __forceinline__ void load_block(double (*A)[DP], const double *V, int n, int k0, int b) {
  for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
    const int r = t & (NB - 1), c = t >> 6;
    A[r][c] = (r < b && c < b) ? V[(size_t)(k0 + r) + (size_t)n * (k0 + c)] : (r == c ? 1.0 : 0.0);
  }
  __syncthreads();
}

// X = A^{-1} for lower-triangular A (both NB x NB in shared memory): row by
// row forward substitution, four threads per column sharing each dot product.
// FP64 arithmetic is scarce on this part, so divisions become one
// reciprocal per row (rdiag, NB doubles of shared memory).
__device__ void tri_inverse(double (*A)[DP], double (*X)[DP], double *part, double *rdiag) {
  const int c = threadIdx.x & (NB - 1), q = threadIdx.x >> 6;  // q = 0..3
  if (threadIdx.x < NB) rdiag[threadIdx.x] = 1.0 / A[threadIdx.x][threadIdx.x];
  __syncthreads();
  for (int r = 0; r < NB; ++r) {
    double s = 0.0;
    for (int p = c + q; p < r; p += 4) s += A[r][p] * X[p][c];
    part[q * NB + c] = s;
    __syncthreads();
    if (q == 0) {
      const double d = (r == c ? 1.0 : 0.0) - (part[c] + part[NB + c] + part[2 * NB + c] +
                                               part[3 * NB + c]);
      X[r][c] = (c <= r) ? d * rdiag[r] : 0.0;
    }
    __syncthreads();
  }
}

// In-place Cholesky of the b x b diagonal block at (k0,k0) of V (ld n) and
// its inverse into Linv (NB x NB, column-major); *bad = pivot+1 on a
// non-positive pivot.
__global__ void __launch_bounds__(256) potrf_inv_block_kernel(double *V, int n, int k0, int b,
                                                             double *Linv, int *bad) {
  extern __shared__ double dsm[];
  double(*A)[DP] = reinterpret_cast<double(*)[DP]>(dsm);
  double(*X)[DP] = reinterpret_cast<double(*)[DP]>(dsm + NB * DP);
  double *part = dsm + 2 * NB * DP;
  double *rdiag = part + 4 * NB;
  double *rpiv = rdiag + NB;
  load_block(A, V, n, k0, b);
  const int c = threadIdx.x & (NB - 1), r0 = threadIdx.x >> 6;
  for (int k = 0; k < NB; ++k) {
    if (threadIdx.x == 0) {
      const double d = A[k][k];
      double l = 1.0;
      if (!(d > 0.0))
        atomicCAS(bad, 0, k0 + k + 1);
      else
        l = sqrt(d);
      A[k][k] = l;
      *rpiv = 1.0 / l;
    }
    __syncthreads();
    if (threadIdx.x > k && threadIdx.x < NB) A[threadIdx.x][k] *= *rpiv;
    __syncthreads();
    // trailing lower triangle: column c, rows r >= c with r = r0 (mod 4)
    if (c > k) {
      const double ck = A[c][k];
      for (int r = c + ((r0 - c) & 3); r < NB; r += 4) A[r][c] -= A[r][k] * ck;
    }
    __syncthreads();
  }
  tri_inverse(A, X, part, rdiag);
  for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
    const int r = t & (NB - 1), cc = t >> 6;
    if (r < b && cc < b) V[(size_t)(k0 + r) + (size_t)n * (k0 + cc)] = (r >= cc) ? A[r][cc] : 0.0;
    Linv[t] = X[r][cc];
  }
}

// Inverses of every diagonal block of the lower-triangular L (one CTA per
// block) into Linv (nblk x NB x NB).
__global__ void __launch_bounds__(256) tri_inverse_blocks_kernel(const double *L, int n,
                                                                double *Linv) {
  extern __shared__ double dsm[];
  double(*A)[DP] = reinterpret_cast<double(*)[DP]>(dsm);
  double(*X)[DP] = reinterpret_cast<double(*)[DP]>(dsm + NB * DP);
  double *part = dsm + 2 * NB * DP;
  double *rdiag = part + 4 * NB;
  const int k0 = blockIdx.x * NB;
  const int b = n - k0 < NB ? n - k0 : NB;
  load_block(A, L, n, k0, b);
  // only the lower triangle of L is meaningful
  for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
    const int r = t & (NB - 1), c = t >> 6;
    if (r < c) A[r][c] = 0.0;
  }
  __syncthreads();
  tri_inverse(A, X, part, rdiag);
  double *out = Linv + (size_t)blockIdx.x * NB * NB;
  for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) out[t] = X[t & (NB - 1)][t >> 6];
}

// The shared-memory opt-in is per device: set it on the current device.
int diag_kernels_init() {
  const bool ok =
      cudaFuncSetAttribute(potrf_inv_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           DIAG_SMEM) == cudaSuccess &&
      cudaFuncSetAttribute(tri_inverse_blocks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           DIAG_SMEM) == cudaSuccess;
  if (!ok) {
    set_error("diagonal-block kernels: shared-memory attribute failed");
    return RIMP2_ERR_CUDA;
  }
  return RIMP2_OK;
}

}  // namespace

// V (n x n, ld n, device) -> lower Cholesky factor in place (strict upper
// zeroed block by block).  Returns RIMP2_ERR_ARG if V is not positive definite.
// Per 64-column block k: factor and invert the diagonal block (one CTA),
// panel P := P L_kk^{-T} as a GEMM with the inverse (into a work panel), the
// trailing update C -= P P^T on the lower-triangle tiles, and the panel
// copied back into V.
int dev_cholesky(int n, double *V, cudaStream_t s) {
  RIMP2_TRY(diag_kernels_init());
  DevBuf bad, inv, panel;
  RIMP2_TRY(bad.alloc(sizeof(int), s));
  RIMP2_TRY(inv.alloc(sizeof(double) * NB * NB, s));
  RIMP2_TRY(panel.alloc(sizeof(double) * (size_t)(n > NB ? n - NB : 1) * NB, s));
  RIMP2_CK(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int b = n - k0 < NB ? n - k0 : NB;
    potrf_inv_block_kernel<<<1, 256, DIAG_SMEM, s>>>(V, n, k0, b, inv.as<double>(),
                                                     bad.as<int>());
    count_launch(1);
    const int rest = n - k0 - b;
    if (rest > 0) {
      double *Pv = V + (size_t)(k0 + b) + (size_t)n * k0;
      {  // panel(rest x b) = P Linv^T
        GemmDesc g = gdesc();
        g.M = rest;
        g.N = b;
        g.K = b;
        g.A = Pv;
        g.sAm = 1;
        g.sAk = n;
        g.B = inv.as<double>();
        g.sBk = NB;
        g.sBn = 1;
        g.C = panel.as<double>();
        g.sCm = 1;
        g.sCn = rest;
        RIMP2_TRY(launch_gemm_f64(g, s));
      }
      {  // trailing update C -= panel panel^T (lower-triangle tiles)
        GemmDesc g = gdesc();
        g.M = rest;
        g.N = rest;
        g.K = b;
        g.alpha = -1.0;
        g.beta = 1.0;
        g.lower = 1;
        g.A = panel.as<double>();
        g.sAm = 1;
        g.sAk = rest;
        g.B = panel.as<double>();
        g.sBk = rest;
        g.sBn = 1;
        g.C = V + (size_t)(k0 + b) + (size_t)n * (k0 + b);
        g.sCm = 1;
        g.sCn = n;
        RIMP2_TRY(launch_gemm_f64(g, s));
      }
      RIMP2_CK(cudaMemcpy2DAsync(Pv, sizeof(double) * n, panel.p, sizeof(double) * rest,
                                 sizeof(double) * rest, b, cudaMemcpyDeviceToDevice, s));
    }
    // zero the strict upper part of this block column above the block
    if (k0 > 0) RIMP2_CK(cudaMemset2DAsync(V + (size_t)n * k0, sizeof(double) * n, 0,
                                           sizeof(double) * k0, b, s));
  }
  RIMP2_CK(cudaGetLastError());
  int h = 0;
  RIMP2_CK(cudaMemcpyAsync(&h, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  RIMP2_CK(cudaStreamSynchronize(s));
  if (h) {
    set_error("auxiliary metric is not positive definite (pivot %d)", h - 1);
    return RIMP2_ERR_ARG;
  }
  return RIMP2_OK;
}

// X = L^{-1} B for B (n x m, ld n).  B is overwritten (used as workspace).
// The inverses of all diagonal blocks come from one launch; then per block
// X_k = inv(L_kk) B_k and B_rest -= L_rest,k X_k (both GEMMs).
int dev_trsm_lower(int n, int m, const double *L, double *B, double *X, cudaStream_t s) {
  RIMP2_TRY(diag_kernels_init());
  const int nblk = (n + NB - 1) / NB;
  DevBuf inv;
  RIMP2_TRY(inv.alloc(sizeof(double) * NB * NB * (size_t)nblk, s));
  tri_inverse_blocks_kernel<<<nblk, 256, DIAG_SMEM, s>>>(L, n, inv.as<double>());
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int b = n - k0 < NB ? n - k0 : NB;
    {  // X_k = inv(L_kk) B_k
      GemmDesc g = gdesc();
      g.M = b;
      g.N = m;
      g.K = b;
      g.A = inv.as<double>() + (size_t)(k0 / NB) * NB * NB;
      g.sAm = 1;
      g.sAk = NB;
      g.B = B + k0;
      g.sBk = 1;
      g.sBn = n;
      g.C = X + k0;
      g.sCm = 1;
      g.sCn = n;
      RIMP2_TRY(launch_gemm_f64(g, s));
    }
    const int rest = n - k0 - b;
    if (rest > 0) {  // B_rest -= L_rest,k X_k
      GemmDesc g = gdesc();
      g.M = rest;
      g.N = m;
      g.K = b;
      g.alpha = -1.0;
      g.beta = 1.0;
      g.A = L + (size_t)(k0 + b) + (size_t)n * k0;
      g.sAm = 1;
      g.sAk = n;
      g.B = X + k0;
      g.sBk = 1;
      g.sBn = n;
      g.C = B + k0 + b;
      g.sCm = 1;
      g.sCn = n;
      RIMP2_TRY(launch_gemm_f64(g, s));
    }
  }
  return RIMP2_OK;
}

// (alpha|a i) from (alpha|mu nu) and the MO coefficients
int dev_ao2mo(int NBA, int nbas, int nocc, int nvirt, const double *ao, const double *Cmo,
              double *out, cudaStream_t s) {
  const long long rows = (long long)NBA * nbas;
  if (rows > 2147483647LL) {
    set_error("ao2mo: NBA*nbas too large");
    return RIMP2_ERR_ARG;
  }
  DevBuf half;
  RIMP2_TRY(half.alloc(sizeof(double) * (size_t)rows * nocc, s));
  {  // half(alpha,mu,i) = sum_nu ao(alpha,mu,nu) Cmo(nu,i)
    GemmDesc g = gdesc();
    g.M = (int)rows;
    g.N = nocc;
    g.K = nbas;
    g.A = ao;
    g.sAm = 1;
    g.sAk = rows;
    g.B = Cmo;
    g.sBk = 1;
    g.sBn = nbas;
    g.C = half.as<double>();
    g.sCm = 1;
    g.sCn = rows;
    RIMP2_TRY(launch_gemm_f64(g, s));
  }
  {  // out(alpha,a,i) = sum_mu half(alpha,mu,i) Cmo(mu,nocc+a)
    GemmDesc g = gdesc();
    g.M = NBA;
    g.N = nvirt;
    g.K = nbas;
    g.A = half.as<double>();
    g.sAm = 1;
    g.sAk = NBA;
    g.sAb0 = rows;
    g.B = Cmo + (size_t)nbas * nocc;
    g.sBk = 1;
    g.sBn = nbas;
    g.C = out;
    g.sCm = 1;
    g.sCn = NBA;
    g.sCb0 = (long long)NBA * nvirt;
    g.nb0 = nocc;
    RIMP2_TRY(launch_gemm_f64(g, s));
  }
  return RIMP2_OK;
}

// (alpha|a i) on the tcgen05 tensor cores with exact-integer FP16 slices
// (S0 + two residual slices, ~2^-33 relative per product): the AO tensor is
// sliced with K = nu contiguous (rows mu + nbas*alpha), contracted with the
// occupied MO columns into half(i, alpha, mu), which is sliced again (rows
// (alpha, i), K = mu) and contracted with the virtual MO columns, written in
// the Calpha layout (alpha, a, i).
int dev_ao2mo_split(int NBA, int nbas, int nocc, int nvirt, const double *ao, const double *Cmo,
                    double *out, cudaStream_t s) {
  const int nsl = 3;
  const long long MK = (long long)NBA * nbas;
  DevBuf half;
  RIMP2_TRY(half.alloc(sizeof(double) * (size_t)MK * nocc, s));
  bool fused = false;
  RIMP2_TRY(ao_half_fused(ao, NBA, nbas, Cmo, nocc, half.as<double>(), s, &fused));
  if (!fused) {
    SlicedOp Aao, Bocc;
    RIMP2_TRY(sliced_ao(Aao, ao, NBA, nbas, nsl, s));
    RIMP2_TRY(sliced_cols(Bocc, Cmo, nbas, nocc, 1, nsl, s));
    // half[i][alpha][mu] = sum_nu ao(alpha,mu,nu) Cmo(nu,i); GEMM row m' = mu + nbas*alpha
    RIMP2_TRY(split_gemm(Aao, 0, 0, Bocc, 0, 0, (int)MK, nocc, 1, half.as<double>(), 1, MK, 0, s));
  }
  SlicedOp Ah, Bv;
  RIMP2_TRY(sliced_cols(Ah, half.as<double>(), nbas, NBA, nocc, nsl, s));
  RIMP2_TRY(sliced_cols(Bv, Cmo + (size_t)nbas * nocc, nbas, nvirt, 1, nsl, s));
  // out(alpha,a,i) = sum_mu half[i][alpha][mu] Cmo(mu,nocc+a)
  RIMP2_TRY(split_gemm(Ah, 0, Ah.rows_per_group, Bv, 0, 0, NBA, nvirt, nocc, out, 1, NBA,
                       (long long)NBA * nvirt, s));
  return RIMP2_OK;
}

int dev_calpha_from_ao(int NBA, int nbas, int nocc, int nvirt, const double *ao, const double *V,
                       const double *Cmo, double *Calpha, cudaStream_t s, bool split_transform) {
  DevBuf L, B;
  RIMP2_TRY(L.alloc(sizeof(double) * (size_t)NBA * NBA, s));
  RIMP2_CK(cudaMemcpyAsync(L.p, V, sizeof(double) * (size_t)NBA * NBA, cudaMemcpyDeviceToDevice, s));
  RIMP2_TRY(dev_cholesky(NBA, L.as<double>(), s));
  RIMP2_TRY(B.alloc(sizeof(double) * (size_t)NBA * nvirt * nocc, s));
  if (split_transform)
    RIMP2_TRY(dev_ao2mo_split(NBA, nbas, nocc, nvirt, ao, Cmo, B.as<double>(), s));
  else
    RIMP2_TRY(dev_ao2mo(NBA, nbas, nocc, nvirt, ao, Cmo, B.as<double>(), s));
  RIMP2_TRY(dev_trsm_lower(NBA, nvirt * nocc, L.as<double>(), B.as<double>(), Calpha, s));
  return RIMP2_OK;
}

}  // namespace rimp2

using namespace rimp2;

extern "C" int rimp2_calpha_from_ao_dev(int NBA, int nbas, int nocc, int nvirt, const double *dao,
                                        const double *dV, const double *dCmo, double *dCalpha,
                                        void *stream) {
  clear_error();
  RIMP2_REQ(NBA > 0 && nbas > 0 && nocc > 0 && nvirt > 0 && nocc + nvirt <= nbas,
            "rimp2_calpha_from_ao_dev: bad dims (need nocc+nvirt <= nbas)");
  RIMP2_REQ(dao && dV && dCmo && dCalpha, "rimp2_calpha_from_ao_dev: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return dev_calpha_from_ao(NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha, s, false);
}

extern "C" int rimp2_ao2mo_dev(int NBA, int nbas, int nocc, int nvirt, const double *dao,
                               const double *dCmo, double *dout, int split, void *stream) {
  clear_error();
  RIMP2_REQ(NBA > 0 && nbas > 0 && nocc > 0 && nvirt > 0 && nocc + nvirt <= nbas,
            "rimp2_ao2mo_dev: bad dims (need nocc+nvirt <= nbas)");
  RIMP2_REQ(dao && dCmo && dout, "rimp2_ao2mo_dev: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return split ? dev_ao2mo_split(NBA, nbas, nocc, nvirt, dao, dCmo, dout, s)
               : dev_ao2mo(NBA, nbas, nocc, nvirt, dao, dCmo, dout, s);
}

extern "C" int rimp2_calpha_from_ao_split_dev(int NBA, int nbas, int nocc, int nvirt,
                                              const double *dao, const double *dV,
                                              const double *dCmo, double *dCalpha, void *stream) {
  clear_error();
  RIMP2_REQ(NBA > 0 && nbas > 0 && nocc > 0 && nvirt > 0 && nocc + nvirt <= nbas,
            "rimp2_calpha_from_ao_split_dev: bad dims (need nocc+nvirt <= nbas)");
  RIMP2_REQ(dao && dV && dCmo && dCalpha, "rimp2_calpha_from_ao_split_dev: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return dev_calpha_from_ao(NBA, nbas, nocc, nvirt, dao, dV, dCmo, dCalpha, s, true);
}

extern "C" int rimp2_calpha_from_ao(const int *NBA, const int *nbas, const int *nocc,
                                    const int *nvirt, const double *ao, const double *V,
                                    const double *Cmo, double *Calpha) {
  clear_error();
  RIMP2_REQ(NBA && nbas && nocc && nvirt && *NBA > 0 && *nbas > 0 && *nocc > 0 && *nvirt > 0 &&
                *nocc + *nvirt <= *nbas,
            "rimp2_calpha_from_ao: bad dims (need nocc+nvirt <= nbas)");
  RIMP2_REQ(ao && V && Cmo && Calpha, "rimp2_calpha_from_ao: null array");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = current_stream();
  const size_t nb = *NBA, n = *nbas;
  DevBuf dao, dV, dC, dOut;
  RIMP2_TRY(dao.alloc(sizeof(double) * nb * n * n, s));
  RIMP2_CK(cudaMemcpyAsync(dao.p, ao, sizeof(double) * nb * n * n, cudaMemcpyHostToDevice, s));
  RIMP2_TRY(dV.alloc(sizeof(double) * nb * nb, s));
  RIMP2_CK(cudaMemcpyAsync(dV.p, V, sizeof(double) * nb * nb, cudaMemcpyHostToDevice, s));
  RIMP2_TRY(dC.alloc(sizeof(double) * n * n, s));
  RIMP2_CK(cudaMemcpyAsync(dC.p, Cmo, sizeof(double) * n * n, cudaMemcpyHostToDevice, s));
  const size_t no = (size_t)nb * *nvirt * *nocc;
  RIMP2_TRY(dOut.alloc(sizeof(double) * no, s));
  RIMP2_TRY(dev_calpha_from_ao(*NBA, *nbas, *nocc, *nvirt, dao.as<double>(), dV.as<double>(),
                               dC.as<double>(), dOut.as<double>(), s, false));
  RIMP2_CK(cudaMemcpyAsync(Calpha, dOut.p, sizeof(double) * no, cudaMemcpyDeviceToHost, s));
  RIMP2_CK(cudaStreamSynchronize(s));
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

extern "C" int rimp2_cholesky_dev(int n, double *dV, void *stream) {
  clear_error();
  RIMP2_REQ(n > 0 && dV, "rimp2_cholesky_dev: bad arguments");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return dev_cholesky(n, dV, s);
}

extern "C" int rimp2_trsm_lower_dev(int n, int m, const double *dL, double *dB, double *dX,
                                    void *stream) {
  clear_error();
  RIMP2_REQ(n > 0 && m > 0 && dL && dB && dX && dB != dX, "rimp2_trsm_lower_dev: bad arguments");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  return dev_trsm_lower(n, m, dL, dB, dX, s);
}
