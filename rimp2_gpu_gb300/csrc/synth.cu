// synth.cu -- seeded synthetic fragments generated on the device.
//
// Counter-based Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) with
// Box-Muller normals, using the same counter layout as the workload
// definition: normal number n of stream s is taken from the uniform pair of
// counter (n/2 lo, n/2 hi, s, 0x5249) under key (seed lo, seed hi), cosine
// branch for even n, sine branch for odd n.
//   Calpha(alpha,a,i) = N(0,1) * 0.03 / sqrt(1 + alpha/64)   (stream 0,
//                        n = column-major linear index of the element)
//   EVocc  sorted U[-1.5,-0.3]  (stream 1),  EVvirt sorted U[0.1,3.0] (stream 2)
// Inputs are created where they are consumed, so a 4 GB fragment costs a few
// milliseconds instead of a host generation plus a PCIe/C2C copy.
#include <cstring>

#include "common.cuh"

namespace rimp2 {
void count_launch(int n);
namespace {

__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ void uniform2(unsigned long long seed, uint32_t stream,
                                         unsigned long long n, double &u0, double &u1) {
  uint32_t c[4] = {(uint32_t)n, (uint32_t)(n >> 32), stream, 0x5249u};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const unsigned long long a = ((unsigned long long)(c[0] >> 5) << 26) | (c[1] >> 6);
  const unsigned long long b = ((unsigned long long)(c[2] >> 5) << 26) | (c[3] >> 6);
  u0 = ((double)a + 0.5) * (1.0 / 9007199254740992.0);
  u1 = ((double)b + 0.5) * (1.0 / 9007199254740992.0);
}

__global__ void gen_calpha_kernel(unsigned long long seed, int NBA, long long total, double *Ca) {
  const long long pair = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = 2 * pair;
  if (n >= total) return;
  double u0, u1;
  uniform2(seed, 0u, (unsigned long long)pair, u0, u1);
  const double r = sqrt(-2.0 * log(u0));
  double sn, cs;
  sincos(6.283185307179586476925286766559 * u1, &sn, &cs);
  const int al0 = (int)(n % NBA);
  Ca[n] = r * cs * 0.03 / sqrt(1.0 + al0 / 64.0);
  if (n + 1 < total) {
    const int al1 = (int)((n + 1) % NBA);
    Ca[n + 1] = r * sn * 0.03 / sqrt(1.0 + al1 / 64.0);
  }
}

// one block: draw, then rank-sort (n is a few thousand at most)
__global__ void gen_eps_kernel(unsigned long long seed, uint32_t stream, int n, double lo,
                               double width, double *out) {
  extern __shared__ double v[];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double u0, u1;
    uniform2(seed, stream, (unsigned long long)(k >> 1), u0, u1);
    v[k] = lo + width * ((k & 1) ? u1 : u0);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double x = v[k];
    int rank = 0;
    for (int m = 0; m < n; ++m) rank += (v[m] < x) || (v[m] == x && m < k);
    out[rank] = x;
  }
}

// (alpha|mu nu) = N(0,1) exp(-|mu-nu|/32), symmetric; normal number
// alpha + NBA*tri(mu<=nu) of stream 3 (tri = nu(nu+1)/2 + mu)
__global__ void gen_ao_kernel(unsigned long long seed, int NBA, int nbas, double *ao) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long ntri = (long long)nbas * (nbas + 1) / 2;
  if (t >= ntri * NBA) return;
  const int al = (int)(t % NBA);
  const long long tri = t / NBA;
  int nu = (int)((sqrt(8.0 * (double)tri + 1.0) - 1.0) * 0.5);
  while ((long long)(nu + 1) * (nu + 2) / 2 <= tri) ++nu;
  while ((long long)nu * (nu + 1) / 2 > tri) --nu;
  const int mu = (int)(tri - (long long)nu * (nu + 1) / 2);
  const unsigned long long n = (unsigned long long)t;  // = al + NBA*tri
  double u0, u1;
  uniform2(seed, 3u, n >> 1, u0, u1);
  const double r = sqrt(-2.0 * log(u0));
  double sn, cs;
  sincos(6.283185307179586476925286766559 * u1, &sn, &cs);
  const double v = ((n & 1) ? r * sn : r * cs) * exp(-fabs((double)(mu - nu)) / 32.0);
  ao[al + (size_t)NBA * (mu + (size_t)nbas * nu)] = v;
  ao[al + (size_t)NBA * (nu + (size_t)nbas * mu)] = v;
}

// N(0,1) matrix of stream `stream`, element n = column-major index
__global__ void gen_normal_kernel(unsigned long long seed, uint32_t stream, long long total,
                                  double scale, double *out) {
  const long long pair = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = 2 * pair;
  if (n >= total) return;
  double u0, u1;
  uniform2(seed, stream, (unsigned long long)pair, u0, u1);
  const double r = sqrt(-2.0 * log(u0));
  double sn, cs;
  sincos(6.283185307179586476925286766559 * u1, &sn, &cs);
  out[n] = r * cs * scale;
  if (n + 1 < total) out[n + 1] = r * sn * scale;
}

__global__ void add_diag_kernel(double *V, int n, double d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) V[(size_t)k * n + k] += d;
}

}  // namespace
}  // namespace rimp2

using namespace rimp2;

extern "C" int rimp2_gen_ao_dev(unsigned long long seed, int NBA, int nbas, double *dao, double *dV,
                                void *stream) {
  clear_error();
  RIMP2_REQ(NBA > 0 && nbas > 0, "rimp2_gen_ao_dev: bad dims");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  if (dao) {
    const long long tot = (long long)nbas * (nbas + 1) / 2 * NBA;
    gen_ao_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(seed, NBA, nbas, dao);
    count_launch(1);
  }
  if (dV) {
    // V = A A^T / NBA + 0.1 I with A ~ N(0,1) (stream 4)
    DevBuf A;
    RIMP2_TRY(A.alloc(sizeof(double) * (size_t)NBA * NBA, s));
    const long long tot = (long long)NBA * NBA;
    gen_normal_kernel<<<(unsigned)((tot / 2 + 256) / 256), 256, 0, s>>>(seed, 4u, tot, 1.0,
                                                                        A.as<double>());
    count_launch(1);
    GemmDesc g;
    memset(&g, 0, sizeof g);
    g.M = NBA;
    g.N = NBA;
    g.K = NBA;
    g.alpha = 1.0 / NBA;
    g.beta = 0.0;
    g.A = A.as<double>();
    g.sAm = 1;
    g.sAk = NBA;
    g.B = A.as<double>();
    g.sBk = NBA;
    g.sBn = 1;
    g.C = dV;
    g.sCm = 1;
    g.sCn = NBA;
    g.nb0 = g.nb1 = 1;
    RIMP2_TRY(launch_gemm_f64(g, s));
    add_diag_kernel<<<(NBA + 255) / 256, 256, 0, s>>>(dV, NBA, 0.1);
    count_launch(1);
  }
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

extern "C" int rimp2_gen_fragment_dev(unsigned long long seed, int nocc, int nvirt, int NBA,
                                      double *dCalpha, double *dEVocc, double *dEVvirt,
                                      void *stream) {
  clear_error();
  RIMP2_REQ(nocc > 0 && nvirt > 0 && NBA > 0, "rimp2_gen_fragment_dev: bad dims");
  RIMP2_REQ(nocc <= 6000 && nvirt <= 6000, "rimp2_gen_fragment_dev: nocc/nvirt above 6000");
  RIMP2_TRY(ensure_device());
  cudaStream_t s = stream ? (cudaStream_t)stream : current_stream();
  if (dCalpha) {
    const long long total = (long long)NBA * nvirt * nocc;
    const long long pairs = (total + 1) / 2;
    gen_calpha_kernel<<<(unsigned)((pairs + 255) / 256), 256, 0, s>>>(seed, NBA, total, dCalpha);
    count_launch(1);
  }
  if (dEVocc) {
    gen_eps_kernel<<<1, 256, sizeof(double) * nocc, s>>>(seed, 1u, nocc, -1.5, 1.2, dEVocc);
    count_launch(1);
  }
  if (dEVvirt) {
    gen_eps_kernel<<<1, 256, sizeof(double) * nvirt, s>>>(seed, 2u, nvirt, 0.1, 2.9, dEVvirt);
    count_launch(1);
  }
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}
