// front_end.cu -- Calpha from AO three-centre integrals, all FP64 on the GPU.
//
//   (alpha|a i) = sum_{mu,nu} Cmo(mu,nocc+a) Cmo(nu,i) (alpha|mu nu)
//   V = L L^T (Cholesky of the auxiliary metric)
//   Calpha(:,a,i) = L^{-1} (:|a i)
// so that sum_alpha Calpha(alpha,a,i) Calpha(alpha,b,j) = (ai|V^{-1}|bj).
// The reference starts from Calpha (RIMP2.F90:48-49); this front end has no
// counterpart there.  Every product runs on the FP64 DMMA GEMM of
// fp64_kernels.cu; the Cholesky and the solve are blocked (64) so that all
// but O(n*64^2) of their work is GEMM:
//   Cholesky: diagonal-block factorisation (one CTA), panel solve, trailing
//             update C -= P P^T;
//   solve:    X_k = inv(L_kk) B_k (explicit 64x64 inverse, GEMM), then
//             B_rest -= L_rest,k X_k.
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

// in-place Cholesky of the b x b diagonal block at (k0,k0) of V (ld n);
// sets *bad = k+1 on a non-positive pivot
__global__ void potrf_block_kernel(double *V, int n, int k0, int b, int *bad) {
  __shared__ double A[NB][NB + 1];
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int r = t % b, c = t / b;
    A[r][c] = V[(size_t)(k0 + r) + (size_t)n * (k0 + c)];
  }
  __syncthreads();
  for (int k = 0; k < b; ++k) {
    if (threadIdx.x == 0) {
      const double d = A[k][k];
      if (!(d > 0.0)) {
        atomicCAS(bad, 0, k0 + k + 1);
        A[k][k] = 1.0;
      } else {
        A[k][k] = sqrt(d);
      }
    }
    __syncthreads();
    const double dk = A[k][k];
    for (int r = k + 1 + threadIdx.x; r < b; r += blockDim.x) A[r][k] /= dk;
    __syncthreads();
    // rank-1 update of the remaining lower triangle
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
      const int r = t % b, c = t / b;
      if (c > k && r >= c) A[r][c] -= A[r][k] * A[c][k];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int r = t % b, c = t / b;
    V[(size_t)(k0 + r) + (size_t)n * (k0 + c)] = (r >= c) ? A[r][c] : 0.0;
  }
}

// rows below the diagonal block: P := P L_kk^{-T}  (one thread per row)
__global__ void panel_solve_kernel(double *V, int n, int k0, int b) {
  __shared__ double L[NB][NB + 1];
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int r = t % b, c = t / b;
    L[r][c] = V[(size_t)(k0 + r) + (size_t)n * (k0 + c)];
  }
  __syncthreads();
  const int row = k0 + b + blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  double x[NB];
  for (int c = 0; c < b; ++c) {
    double s = V[(size_t)row + (size_t)n * (k0 + c)];
    for (int p = 0; p < c; ++p) s -= x[p] * L[c][p];
    x[c] = s / L[c][c];
  }
  for (int c = 0; c < b; ++c) V[(size_t)row + (size_t)n * (k0 + c)] = x[c];
}

// inverse of the lower-triangular b x b block at (k0,k0) of L (ld n) into
// Linv (b x b, ld NB): one thread per column, forward substitution
__global__ void trinv_block_kernel(const double *L, int n, int k0, int b, double *Linv) {
  __shared__ double A[NB][NB + 1];
  for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
    const int r = t % b, c = t / b;
    A[r][c] = L[(size_t)(k0 + r) + (size_t)n * (k0 + c)];
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c >= NB) return;
  double x[NB];
  for (int r = 0; r < NB; ++r) {
    double v = 0.0;
    if (c < b && r < b && r >= c) {
      double s = (r == c) ? 1.0 : 0.0;
      for (int p = c; p < r; ++p) s -= A[r][p] * x[p];
      v = s / A[r][r];
    }
    x[r] = v;
  }
  for (int r = 0; r < NB; ++r) Linv[r + NB * c] = x[r];
}

}  // namespace

// V (n x n, ld n, device) -> lower Cholesky factor in place (strict upper
// zeroed block by block).  Returns RIMP2_ERR_ARG if V is not positive definite.
int dev_cholesky(int n, double *V, cudaStream_t s) {
  DevBuf bad;
  RIMP2_TRY(bad.alloc(sizeof(int), s));
  RIMP2_CK(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int b = n - k0 < NB ? n - k0 : NB;
    potrf_block_kernel<<<1, 256, 0, s>>>(V, n, k0, b, bad.as<int>());
    count_launch(1);
    const int rest = n - k0 - b;
    if (rest > 0) {
      panel_solve_kernel<<<(rest + 127) / 128, 128, 0, s>>>(V, n, k0, b);
      count_launch(1);
      // trailing update C -= P P^T on the whole trailing square
      GemmDesc g = gdesc();
      g.M = rest;
      g.N = rest;
      g.K = b;
      g.alpha = -1.0;
      g.beta = 1.0;
      g.A = V + (size_t)(k0 + b) + (size_t)n * k0;
      g.sAm = 1;
      g.sAk = n;
      g.B = g.A;
      g.sBk = n;
      g.sBn = 1;
      g.C = V + (size_t)(k0 + b) + (size_t)n * (k0 + b);
      g.sCm = 1;
      g.sCn = n;
      RIMP2_TRY(launch_gemm_f64(g, s));
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
int dev_trsm_lower(int n, int m, const double *L, double *B, double *X, cudaStream_t s) {
  DevBuf inv;
  RIMP2_TRY(inv.alloc(sizeof(double) * NB * NB, s));
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int b = n - k0 < NB ? n - k0 : NB;
    trinv_block_kernel<<<1, NB, 0, s>>>(L, n, k0, b, inv.as<double>());
    count_launch(1);
    {  // X_k = inv(L_kk) B_k
      GemmDesc g = gdesc();
      g.M = b;
      g.N = m;
      g.K = b;
      g.A = inv.as<double>();
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
  {
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
