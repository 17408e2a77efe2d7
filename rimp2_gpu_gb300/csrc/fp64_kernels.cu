// fp64_kernels.cu -- FP64 kernels on the DMMA (mma.sync .f64) tensor path.
//
//  * gemm_f64_kernel: strided, batched column-major-agnostic FP64 contraction
//    C(m,n) = alpha * sum_k A(m,k) B(k,n) + beta * C(m,n) with an optional
//    orbital-energy denominator epilogue.  It carries every FP64 product of
//    the drop-in subroutines (toccA/tvirtA g/D and projections, toccB/tvirtB,
//    TransAlpha1/2, gocc/gvirt/gen4DimFO, the driver's DGEMMs).
//  * the fused FP64 energy: a work item is the tile pair (A,B) of occupied
//    pair (i<=j): T1 = G_ij[A,B] = C_iA^T C_jB and T2 = G_ji[A,B] =
//    C_jA^T C_iB share the (a,b) layout, so the exchange integral g_ij(b,a)
//    sits in the same thread as g_ij(a,b) and the four-index integrals never
//    leave the chip.  plain_batch_kernel is the persistent form (a queue of
//    items over one or many fragments, the energy path); plain_energy_kernel
//    runs one item per CTA and can also write the amplitude array.
//  * eos_energy_kernel: the same items with a second, projected Calpha (the
//    local-orbital fragment energy).
//
// GB300 FP64 throughput is a small fraction of its low-precision tensor
// rate, so these kernels are arithmetic-bound by construction: shared-memory
// staging is simple (cp.async double buffering in the GEMM), padding keeps
// fragment loads bank-conflict free, and two CTAs per SM keep the FP64 pipe
// busy.
#include "common.cuh"

#include <algorithm>
#include <vector>

namespace rimp2 {

namespace {

constexpr int TM = 64;   // CTA tile rows
constexpr int TN = 64;   // CTA tile cols
constexpr int TK = 16;   // K slab
constexpr int KP = 20;   // padded slab row (doubles): conflict-free 8x4 fragment reads
constexpr int NTHR = 256;

// D(8x8) += A(8x4, row) * B(4x8, col), FP64 tensor op.
// Fragments: a = A[lane>>2][lane&3], b = B[lane&3][lane>>2],
// d0/d1 = D[lane>>2][2*(lane&3) + 0/1].
__device__ __forceinline__ void dmma884(double &d0, double &d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// ---------------------------------------------------------------------------
// Generic strided batched GEMM
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async8(double *dst, const double *src, bool valid) {
  // 8-byte global -> shared copy; an invalid element is zero-filled (no read)
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src),
               "r"(valid ? 8 : 0)
               : "memory");
}

// The 16-wide K slabs are double-buffered with cp.async: the next slab is in
// flight while the DMMA loop consumes the current one.
__global__ void __launch_bounds__(NTHR) gemm_f64_kernel(GemmDesc g) {
  __shared__ double As[2][TM][KP];
  __shared__ double Bs[2][TN][KP];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
  const int gid = lane >> 2, tig = lane & 3;
  const bool a_kcontig = (g.sAk == 1);
  const bool b_kcontig = (g.sBk == 1);
  const long long nbat = (long long)g.nb0 * g.nb1;

  for (long long bz = blockIdx.z; bz < nbat; bz += gridDim.z) {
    const int b0 = (int)(bz % g.nb0), b1 = (int)(bz / g.nb0);
    const double *Ab = g.A + b0 * g.sAb0 + b1 * g.sAb1;
    const double *Bb = g.B + b0 * g.sBb0 + b1 * g.sBb1;
    double *Cb = g.C + b0 * g.sCb0 + b1 * g.sCb1;
    for (int by = blockIdx.y; by * TN < g.N; by += gridDim.y) {
      const int m0 = blockIdx.x * TM, n0 = by * TN;
      if (g.lower && n0 > m0 + TM - 1) continue;  // tile strictly above the diagonal
      double acc[4][2][2];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) acc[x][y][0] = acc[x][y][1] = 0.0;

      // stage A(m0:m0+64, k0:k0+16) and B(k0:k0+16, n0:n0+64) into buffer buf
      auto load_slab = [&](int buf, int k0) {
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          int mm, kk;
          if (a_kcontig) {
            kk = tid & 15;
            mm = (tid >> 4) + 16 * p;
          } else {
            mm = tid & 63;
            kk = (tid >> 6) + 4 * p;
          }
          const int m = m0 + mm, k = k0 + kk;
          const bool va = (m < g.M && k < g.K);
          cp_async8(&As[buf][mm][kk], va ? Ab + (long long)m * g.sAm + (long long)k * g.sAk : Ab,
                    va);
          int nn, kb;
          if (b_kcontig) {
            kb = tid & 15;
            nn = (tid >> 4) + 16 * p;
          } else {
            nn = tid & 63;
            kb = (tid >> 6) + 4 * p;
          }
          const int n = n0 + nn, kq = k0 + kb;
          const bool vb = (n < g.N && kq < g.K);
          cp_async8(&Bs[buf][nn][kb], vb ? Bb + (long long)kq * g.sBk + (long long)n * g.sBn : Bb,
                    vb);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
      };

      if (g.K > 0) load_slab(0, 0);
      int cur = 0;
      for (int k0 = 0; k0 < g.K; k0 += TK, cur ^= 1) {
        if (k0 + TK < g.K) {
          load_slab(cur ^ 1, k0 + TK);
          asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < TK; ks += 4) {
          double af[4], bf[2];
#pragma unroll
          for (int x = 0; x < 4; ++x) af[x] = As[cur][wm + 8 * x + gid][ks + tig];
#pragma unroll
          for (int y = 0; y < 2; ++y) bf[y] = Bs[cur][wn + 8 * y + gid][ks + tig];
#pragma unroll
          for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 2; ++y) dmma884(acc[x][y][0], acc[x][y][1], af[x], bf[y]);
        }
        __syncthreads();  // buffer cur is refilled two slabs later
      }
      // epilogue
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int m = m0 + wm + 8 * x + gid;
            const int n = n0 + wn + 8 * y + 2 * tig + h;
            if (m < g.M && n < g.N) {
              double v = acc[x][y][h];
              if (g.denom == 1) {
                // RIMP2.F90:403-404: deltaEPS = EVocc(I)+EVocc(J)-EVvirt(B)-EVvirt(A)
                const double d = g.eo[b0] + g.eo[b1] - g.ev[n] - g.ev[m];
                v = v / d;
              }
              double *cp = Cb + m * g.sCm + n * g.sCn;
              v = g.alpha * v;
              if (g.beta != 0.0) v += g.beta * *cp;
              *cp = v;
            }
          }
    }
  }
}

// ---------------------------------------------------------------------------
// Fused FP64 energy kernel
// ---------------------------------------------------------------------------
__device__ __forceinline__ void decode_tri(int q, int &A, int &B) {
  // q = B*(B+1)/2 + A, 0 <= A <= B
  int b = (int)((sqrt(8.0 * q + 1.0) - 1.0) * 0.5);
  while ((b + 1) * (b + 2) / 2 <= q) ++b;
  while (b * (b + 1) / 2 > q) --b;
  B = b;
  A = q - b * (b + 1) / 2;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Accumulate T1 = C_iA^T C_jB and T2 = C_jA^T C_iB (64x64 each, FP64 DMMA)
// over the whole K = NBA for the tile pair at (a0, b0); i = j skips T2.
// Fragment ownership: warp w holds rows wm + 8x + gid, columns wn + 8y + 2 tig + h.
__device__ __forceinline__ void accumulate_tile_pair(double (&P)[4][TM][KP],
                                                     const double *__restrict__ Ca, int NBA,
                                                     int nvirt, int i, int j, int a0, int b0,
                                                     double (&t1)[4][2][2],
                                                     double (&t2)[4][2][2]) {
  const bool same = (i == j);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
  const int gid = lane >> 2, tig = lane & 3;
  const size_t colstride = (size_t)NBA;
  const double *ci = Ca + (size_t)NBA * nvirt * i;
  const double *cj = Ca + (size_t)NBA * nvirt * j;
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y) t1[x][y][0] = t1[x][y][1] = t2[x][y][0] = t2[x][y][1] = 0.0;

  for (int k0 = 0; k0 < NBA; k0 += TK) {
    const int kk = tid & 15;
    const int k = k0 + kk;
#pragma unroll
    for (int pp = 0; pp < 4; ++pp) {
      const int cc = (tid >> 4) + 16 * pp;  // column within tile
      const int a = a0 + cc, b = b0 + cc;
      const bool ka = (k < NBA);
      P[0][cc][kk] = (ka && a < nvirt) ? ci[a * colstride + k] : 0.0;
      P[1][cc][kk] = (ka && b < nvirt) ? cj[b * colstride + k] : 0.0;
      if (!same) {
        P[2][cc][kk] = (ka && a < nvirt) ? cj[a * colstride + k] : 0.0;
        P[3][cc][kk] = (ka && b < nvirt) ? ci[b * colstride + k] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < TK; ks += 4) {
      double a1[4], b1[2];
#pragma unroll
      for (int x = 0; x < 4; ++x) a1[x] = P[0][wm + 8 * x + gid][ks + tig];
#pragma unroll
      for (int y = 0; y < 2; ++y) b1[y] = P[1][wn + 8 * y + gid][ks + tig];
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) dmma884(t1[x][y][0], t1[x][y][1], a1[x], b1[y]);
      if (!same) {
        double a2[4], b2[2];
#pragma unroll
        for (int x = 0; x < 4; ++x) a2[x] = P[2][wm + 8 * x + gid][ks + tig];
#pragma unroll
        for (int y = 0; y < 2; ++y) b2[y] = P[3][wn + 8 * y + gid][ks + tig];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 2; ++y) dmma884(t2[x][y][0], t2[x][y][1], a2[x], b2[y]);
      }
    }
    __syncthreads();
  }

}

// Energy contribution of tile pair (tA,tB) of occupied pair (i<=j); the
// block sum is valid in thread 0.  Shared staging P and red are the caller's.
__device__ __forceinline__ double plain_tile_pair(double (&P)[4][TM][KP], double *red,
                                                  const double *__restrict__ Ca, int NBA,
                                                  int nvirt, int nocc,
                                                  const double *__restrict__ eo,
                                                  const double *__restrict__ ev, int i, int j,
                                                  int tA, int tB, double *__restrict__ tamp) {
  const bool same = (i == j);
  const int a0 = tA * TM, b0 = tB * TN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
  const int gid = lane >> 2, tig = lane & 3;

  double t1[4][2][2], t2[4][2][2];
  accumulate_tile_pair(P, Ca, NBA, nvirt, i, j, a0, b0, t1, t2);

  // epilogue: denominators, amplitudes, energy contribution
  const double eij = eo[i] + eo[j];
  const bool diag = (tA == tB);
  double e = 0.0;
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int a = a0 + wm + 8 * x + gid;
        const int b = b0 + wn + 8 * y + 2 * tig + h;
        if (a < nvirt && b < nvirt) {
          const double g1 = t1[x][y][h];
          const double g2 = same ? g1 : t2[x][y][h];
          const double d = eij - ev[b] - ev[a];  // RIMP2.F90:403 order
          const double u1 = g1 / d, u2 = g2 / d;
          e += u1 * (2.0 * g1 - g2);
          if (!diag) e += u2 * (2.0 * g2 - g1);
          if (tamp) {
            // t(a,i,b,j) = g_ij(a,b)/D ; t(b,i,a,j) = g_ij(b,a)/D
            // t(a,j,b,i) = g_ji(a,b)/D = g_ij(b,a)/D ; t(b,j,a,i) = g_ij(a,b)/D
            const size_t nv = nvirt, no = nocc;
            tamp[a + nv * (i + no * (b + nv * j))] = u1;
            if (!diag) tamp[b + nv * (i + no * (a + nv * j))] = u2;
            if (!same) {
              tamp[a + nv * (j + no * (b + nv * i))] = u2;
              if (!diag) tamp[b + nv * (j + no * (a + nv * i))] = u1;
            }
          }
        }
      }
  e = warp_sum(e);
  if (lane == 0) red[warp] = e;
  __syncthreads();
  double s = 0.0;
  if (tid == 0)
    for (int w = 0; w < NTHR / 32; ++w) s += red[w];
  return s;
}

// part[item] = contribution of tile pair (A,B) to e_ij of pair p
__global__ void __launch_bounds__(NTHR, 2) plain_energy_kernel(const double *__restrict__ Ca, int NBA,
                                                            int nvirt, int nocc,
                                                            const double *__restrict__ eo,
                                                            const double *__restrict__ ev,
                                                            const int *__restrict__ pairs,
                                                            int ntile, double *__restrict__ part,
                                                            double *__restrict__ tamp) {
  __shared__ double P[4][TM][KP];  // C_iA, C_jB, C_jA, C_iB slabs
  __shared__ double red[NTHR / 32];
  const int ntp = ntile * (ntile + 1) / 2;
  const long long item = blockIdx.x;
  const int p = (int)(item / ntp), q = (int)(item % ntp);
  int tA, tB;
  decode_tri(q, tA, tB);
  const double s = plain_tile_pair(P, red, Ca, NBA, nvirt, nocc, eo, ev, pairs[2 * p],
                                   pairs[2 * p + 1], tA, tB, tamp);
  if (threadIdx.x == 0) part[item] = s;
}

// Fragment energy with local orbitals, fused: for Calpha C and its projected
// copy Ct (both (NBA,nvirt,nocc)), tile pair (tA,tB) of pair (i<=j) adds
//   sum_(a,b) g_ij^ab / D * (2 gt_ij^ab - gt_ij^ba)
// over (a in A, b in B) and, off the diagonal tile pair, (a in B, b in A),
// where g comes from C and gt from Ct.  T1/T2 of C are accumulated first and
// parked in a thread-private shared-memory stash (each thread reads back only
// what it wrote), then T1/T2 of Ct; registers stay at the plain kernel's.
constexpr int EOS_STASH = 32;  // doubles per thread
constexpr int EOS_SMEM = (4 * TM * KP + EOS_STASH * NTHR + NTHR / 32) * (int)sizeof(double);

__global__ void __launch_bounds__(NTHR, 2) eos_energy_kernel(const double *__restrict__ Ca,
                                                             const double *__restrict__ Ct,
                                                             int NBA, int nvirt,
                                                             const double *__restrict__ eo,
                                                             const double *__restrict__ ev,
                                                             const int *__restrict__ pairs,
                                                             int ntile, double *__restrict__ part) {
  extern __shared__ double esm[];
  double(&P)[4][TM][KP] = *reinterpret_cast<double(*)[4][TM][KP]>(esm);
  double *stash = esm + 4 * TM * KP;          // [EOS_STASH][NTHR]
  double *red = stash + EOS_STASH * NTHR;     // [NTHR / 32]
  const int ntp = ntile * (ntile + 1) / 2;
  const long long item = blockIdx.x;
  const int p = (int)(item / ntp), q = (int)(item % ntp);
  int tA, tB;
  decode_tri(q, tA, tB);
  const int i = pairs[2 * p], j = pairs[2 * p + 1];
  const bool same = (i == j), diag = (tA == tB);
  const int a0 = tA * TM, b0 = tB * TN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
  const int gid = lane >> 2, tig = lane & 3;

  double t1[4][2][2], t2[4][2][2];
  accumulate_tile_pair(P, Ca, NBA, nvirt, i, j, a0, b0, t1, t2);
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = (x * 2 + y) * 2 + h;
        stash[(2 * r) * NTHR + tid] = t1[x][y][h];
        stash[(2 * r + 1) * NTHR + tid] = same ? t1[x][y][h] : t2[x][y][h];
      }
  accumulate_tile_pair(P, Ct, NBA, nvirt, i, j, a0, b0, t1, t2);  // now gt

  const double eij = eo[i] + eo[j];
  double e = 0.0;
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int a = a0 + wm + 8 * x + gid;
        const int b = b0 + wn + 8 * y + 2 * tig + h;
        if (a < nvirt && b < nvirt) {
          const int r = (x * 2 + y) * 2 + h;
          const double g1 = stash[(2 * r) * NTHR + tid], g2 = stash[(2 * r + 1) * NTHR + tid];
          const double u1 = t1[x][y][h], u2 = same ? u1 : t2[x][y][h];
          const double d = eij - ev[b] - ev[a];  // RIMP2.F90:403 order
          e += g1 / d * (2.0 * u1 - u2);
          if (!diag) e += g2 / d * (2.0 * u2 - u1);
        }
      }
  e = warp_sum(e);
  if (lane == 0) red[warp] = e;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < NTHR / 32; ++w) s += red[w];
    part[item] = s;
  }
}

// Batched form: one persistent launch drains a queue of (fragment, pair,
// tile pair) items over every fragment of the batch.  Fragments are ordered
// heaviest first (by NBA, the K length of each item), so the long items lead
// the queue and the short ones fill the tail.
__device__ __forceinline__ void decode_pair_ij(int p, int &i, int &j) {
  // p = j*(j+1)/2 + i, 0 <= i <= j
  int jj = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
  while ((jj + 1) * (jj + 2) / 2 <= p) ++jj;
  while (jj * (jj + 1) / 2 > p) --jj;
  j = jj;
  i = p - jj * (jj + 1) / 2;
}

__global__ void __launch_bounds__(NTHR) plain_batch_kernel(const PlainFrag *__restrict__ fr,
                                                           int nfrag, long long nitems,
                                                           unsigned int *queue,
                                                           double *__restrict__ part) {
  __shared__ double P[4][TM][KP];
  __shared__ double red[NTHR / 32];
  __shared__ long long s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (long long)atomicAdd(queue, 1u);
    __syncthreads();
    const long long item = s_item;
    if (item >= nitems) break;
    int lo = 0, hi = nfrag - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (fr[mid].item_base <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const PlainFrag &F = fr[lo];
    const long long loc = item - F.item_base;
    int i, j, tA, tB;
    decode_pair_ij((int)(loc / F.ntp), i, j);
    decode_tri((int)(loc % F.ntp), tA, tB);
    const double s = plain_tile_pair(P, red, F.Ca, F.NBA, F.nvirt, F.nocc, F.eo, F.ev, i, j, tA,
                                     tB, nullptr);
    if (threadIdx.x == 0) part[item] = s;
    __syncthreads();  // s_item and red are rewritten by the next item
  }
}

}  // namespace

// Compensated reductions (deterministic: fixed assignment and fixed tree).
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void warp_sum_comp(double &s, double &c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_xor_sync(0xffffffffu, s, o);
    const double c2 = __shfl_xor_sync(0xffffffffu, c, o);
    double t, e;
    // order the operands so every lane combines the same way
    if ((threadIdx.x & o) == 0)
      two_sum(s, s2, t, e);
    else
      two_sum(s2, s, t, e);
    s = t;
    c = ((threadIdx.x & o) == 0 ? c + c2 : c2 + c) + e;
  }
}

// one warp per pair: Epair(i,j) = Epair(j,i) = compensated sum of its items
__global__ void pair_reduce_kernel(const double *__restrict__ part, int nper, const int *pairs,
                                   int npairs, int nocc, double *Epair) {
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= npairs) return;
  double s = 0.0, c = 0.0;
  for (int r = lane; r < nper; r += 32) {
    double t, e;
    two_sum(s, part[(size_t)p * nper + r], t, e);
    s = t;
    c += e;
  }
  warp_sum_comp(s, c);
  if (lane == 0) {
    const double v = s + c;
    const int i = pairs[2 * p], j = pairs[2 * p + 1];
    Epair[i + (size_t)nocc * j] = v;
    Epair[j + (size_t)nocc * i] = v;
  }
}

// Etot = sum_ij Epair(i,j): one block, compensated tree
__device__ __forceinline__ void total_reduce_body(const double *Epair, int nocc, double *Etot) {
  __shared__ double ss[32], sc[32];
  double s = 0.0, c = 0.0;
  const size_t n = (size_t)nocc * nocc;
  for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
    double t, e;
    two_sum(s, Epair[k], t, e);
    s = t;
    c += e;
  }
  warp_sum_comp(s, c);
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
    warp_sum_comp(s, c);
    if (lane == 0) *Etot = s + c;
  }
}

__global__ void total_reduce_kernel(const double *Epair, int nocc, double *Etot) {
  total_reduce_body(Epair, nocc, Etot);
}

__global__ void make_pairs_kernel(int nocc, int *pairs) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = nocc * (nocc + 1) / 2;
  if (n >= np) return;
  int j = (int)((sqrt(8.0 * n + 1.0) - 1.0) * 0.5);
  while ((j + 1) * (j + 2) / 2 <= n) ++j;
  while (j * (j + 1) / 2 > n) --j;
  pairs[2 * n] = n - j * (j + 1) / 2;
  pairs[2 * n + 1] = j;
}

// one warp per (fragment, pair) of a plain batch
__global__ void pair_reduce_plain_batch_kernel(const PlainFrag *__restrict__ fr, int nfrag,
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
  const PlainFrag &F = fr[lo];
  const int p = gp - F.pair_base;
  const double *src = part + F.item_base + (long long)p * F.ntp;
  double s = 0.0, c = 0.0;
  for (int r = lane; r < F.ntp; r += 32) {
    double t, e;
    two_sum(s, src[r], t, e);
    s = t;
    c += e;
  }
  warp_sum_comp(s, c);
  if (lane == 0) {
    int i, j;
    decode_pair_ij(p, i, j);
    const double v = s + c;
    F.Epair[i + (size_t)F.nocc * j] = v;
    F.Epair[j + (size_t)F.nocc * i] = v;
  }
}

// one block per fragment of a plain batch: Etot_f = sum_ij Epair_f(i,j)
__global__ void total_reduce_plain_batch_kernel(const PlainFrag *__restrict__ fr) {
  const PlainFrag &F = fr[blockIdx.x];
  total_reduce_body(F.Epair, F.nocc, F.Etot);
}

void count_launch(int n);

// FP64 tensor-op throughput probe: independent m8n8k4 DMMA chains, used to
// report the plain kernel against the measured FP64 peak of this GPU.
__global__ void dmma_probe_kernel(double *out, int iters) {
  double d[8][2];
  const double a = threadIdx.x * 1e-3, b = 1.0000001;
#pragma unroll
  for (int x = 0; x < 8; ++x) d[x][0] = d[x][1] = 0.0;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int x = 0; x < 8; ++x) dmma884(d[x][0], d[x][1], a, b);
  double r = 0.0;
#pragma unroll
  for (int x = 0; x < 8; ++x) r += d[x][0] + d[x][1];
  if (r == 1234.5) out[0] = r;  // keeps the chains live
}

int probe_fp64_peak(double *tflops, cudaStream_t s) {
  int dev = 0, nsm = 0;
  RIMP2_CK(cudaGetDevice(&dev));
  RIMP2_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  DevBuf o;
  RIMP2_TRY(o.alloc(64, s));
  const int blocks = nsm * 4, thr = 256;
  cudaEvent_t e0, e1;
  RIMP2_CK(cudaEventCreate(&e0));
  RIMP2_CK(cudaEventCreate(&e1));
  // a short calibration launch, then one launch sized to run for at least a
  // second, so that the rate is the one the FP64 pipe sustains at the clock
  // the GPU settles to under this load (a few-ms burst reads higher)
  int iters = 512;
  float ms = 0.f;
  for (int pass = 0; pass < 2; ++pass) {
    RIMP2_CK(cudaEventRecord(e0, s));
    dmma_probe_kernel<<<blocks, thr, 0, s>>>(o.as<double>(), iters);
    RIMP2_CK(cudaEventRecord(e1, s));
    count_launch(1);
    RIMP2_CK(cudaEventSynchronize(e1));
    RIMP2_CK(cudaEventElapsedTime(&ms, e0, e1));
    if (pass == 0) {
      const double scale = 1100.0 / (ms > 0.01f ? ms : 0.01f);
      iters = (int)std::min(2.0e9 / 8.0, std::max(512.0, iters * scale));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // 8 chains x iters x (8x8x4 MACs per warp) x 2 FLOP
  const double flop = 2.0 * 256.0 * 8.0 * iters * ((double)blocks * thr / 32.0);
  *tflops = flop / (ms * 1e-3) / 1e12;
  return RIMP2_OK;
}

int launch_gemm_f64(const GemmDesc &g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.nb0 <= 0 || g.nb1 <= 0) return RIMP2_OK;
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  long long mt = (g.M + TM - 1) / TM, nt = (g.N + TN - 1) / TN;
  long long nb = (long long)g.nb0 * g.nb1;
  if (mt > 2147483647LL) {
    set_error("gemm M too large");
    return RIMP2_ERR_ARG;
  }
  dim3 grid((unsigned)mt, (unsigned)(nt < 65535 ? nt : 65535), (unsigned)(nb < 65535 ? nb : 65535));
  if (g.K <= 0) {
    // C = beta*C (alpha*0): still run the kernel (it handles K=0 as zero sum)
  }
  gemm_f64_kernel<<<grid, NTHR, 0, s>>>(g);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

// Same launches as plain_energy_f64, with the pair list and the per-item
// partials in caller-provided device scratch instead of stream-ordered
// allocations.  pairs_scratch holds 2*npairs ints, part_scratch
// npairs*ntp doubles (plain_energy_scratch_sizes gives both).
void plain_energy_scratch_sizes(int nvirt, int nocc, long long *npairs, long long *nitems) {
  const int ntile = (nvirt + TM - 1) / TM;
  const long long ntp = (long long)ntile * (ntile + 1) / 2;
  *npairs = (long long)nocc * (nocc + 1) / 2;
  *nitems = *npairs * ntp;
}

// Loads the four kernels plain_energy_f64_scratch launches onto the current
// device.  Under CUDA's lazy module loading a kernel's code is placed in
// device memory at its first launch; asking for its attributes loads it now,
// so a later allocation-free call does not need device memory for code.
int preload_plain_scratch_kernels() {
  cudaFuncAttributes fa;
  RIMP2_CK(cudaFuncGetAttributes(&fa, make_pairs_kernel));
  RIMP2_CK(cudaFuncGetAttributes(&fa, plain_energy_kernel));
  RIMP2_CK(cudaFuncGetAttributes(&fa, pair_reduce_kernel));
  RIMP2_CK(cudaFuncGetAttributes(&fa, total_reduce_kernel));
  return RIMP2_OK;
}

int plain_energy_f64_scratch(const PlainEnergyArgs &a, int *pairs_scratch, double *part_scratch,
                             cudaStream_t s) {
  const int ntile = (a.nvirt + TM - 1) / TM;
  const int ntp = ntile * (ntile + 1) / 2;
  const int npairs = a.nocc * (a.nocc + 1) / 2;
  const long long nitems = (long long)npairs * ntp;
  make_pairs_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(a.nocc, pairs_scratch);
  RIMP2_CK(cudaMemsetAsync(a.Epair, 0, sizeof(double) * (size_t)a.nocc * a.nocc, s));
  plain_energy_kernel<<<(unsigned)nitems, NTHR, 0, s>>>(a.Ca, a.NBA, a.nvirt, a.nocc, a.eo, a.ev,
                                                        pairs_scratch, ntile, part_scratch,
                                                        a.tamp);
  pair_reduce_kernel<<<(npairs + 7) / 8, 256, 0, s>>>(part_scratch, ntp, pairs_scratch, npairs,
                                                     a.nocc, a.Epair);
  total_reduce_kernel<<<1, 1024, 0, s>>>(a.Epair, a.nocc, a.Etot);
  count_launch(4);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

int plain_energy_f64(const PlainEnergyArgs &a, cudaStream_t s) {
  if (!a.tamp && !a.pairs) {
    // energies only, all pairs: the persistent form (one launch draining the
    // queue of (pair, tile pair) items, as for a batch of one fragment)
    PlainFrag F;
    memset(&F, 0, sizeof F);
    F.Ca = a.Ca;
    F.eo = a.eo;
    F.ev = a.ev;
    F.Epair = a.Epair;
    F.Etot = a.Etot;
    F.nocc = a.nocc;
    F.nvirt = a.nvirt;
    F.NBA = a.NBA;
    PlainPlan *P = nullptr;
    RIMP2_TRY(plain_plan_create(&P, 1, &F, s));
    const int rc = plain_plan_record(P, s);
    plain_plan_destroy(P);  // workspace is released stream-ordered
    return rc;
  }
  const int ntile = (a.nvirt + TM - 1) / TM;
  const int ntp = ntile * (ntile + 1) / 2;
  const int npairs = a.pairs ? a.npairs : a.nocc * (a.nocc + 1) / 2;
  DevBuf pairs_buf, part;
  const int *pairs = a.pairs;
  if (!pairs) {
    RIMP2_TRY(pairs_buf.alloc(sizeof(int) * 2 * (size_t)npairs, s));
    make_pairs_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(a.nocc, pairs_buf.as<int>());
    count_launch(1);
    RIMP2_CK(cudaGetLastError());
    pairs = pairs_buf.as<int>();
  }
  const long long nitems = (long long)npairs * ntp;
  if (nitems > 2147483647LL) {
    set_error("too many work items (%lld)", nitems);
    return RIMP2_ERR_ARG;
  }
  RIMP2_TRY(part.alloc(sizeof(double) * (size_t)nitems, s));
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  RIMP2_CK(cudaMemsetAsync(a.Epair, 0, sizeof(double) * (size_t)a.nocc * a.nocc, s));
  plain_energy_kernel<<<(unsigned)nitems, NTHR, 0, s>>>(a.Ca, a.NBA, a.nvirt, a.nocc, a.eo, a.ev,
                                                        pairs, ntile, part.as<double>(), a.tamp);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  pair_reduce_kernel<<<(npairs + 7) / 8, 256, 0, s>>>(part.as<double>(), ntp, pairs, npairs, a.nocc,
                                                     a.Epair);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  total_reduce_kernel<<<1, 1024, 0, s>>>(a.Epair, a.nocc, a.Etot);
  count_launch(1);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}


// Fused local-orbital fragment energy: Epair(i,j) = sum_ab g_ij^ab/D (2 gt_ij^ab
// - gt_ij^ba) from Calpha and its projected copy Ct; Etot = sum_ij Epair.
int eos_energy_f64(const double *Ca, const double *Ct, int NBA, int nvirt, int nocc,
                   const double *eo, const double *ev, double *Epair, double *Etot,
                   cudaStream_t s) {
  static_assert(EOS_SMEM <= 227 * 1024, "EOS kernel shared memory");
  const int ntile = (nvirt + TM - 1) / TM;
  const int ntp = ntile * (ntile + 1) / 2;
  const int npairs = nocc * (nocc + 1) / 2;
  const long long nitems = (long long)npairs * ntp;
  if (nitems > 2147483647LL) {
    set_error("too many work items (%lld)", nitems);
    return RIMP2_ERR_ARG;
  }
  RIMP2_CK(cudaFuncSetAttribute(eos_energy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                EOS_SMEM));
  DevBuf pairs, part;
  RIMP2_TRY(pairs.alloc(sizeof(int) * 2 * (size_t)npairs, s));
  RIMP2_TRY(part.alloc(sizeof(double) * (size_t)nitems, s));
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  make_pairs_kernel<<<(npairs + 255) / 256, 256, 0, s>>>(nocc, pairs.as<int>());
  RIMP2_CK(cudaMemsetAsync(Epair, 0, sizeof(double) * (size_t)nocc * nocc, s));
  eos_energy_kernel<<<(unsigned)nitems, NTHR, EOS_SMEM, s>>>(Ca, Ct, NBA, nvirt, eo, ev,
                                                              pairs.as<int>(), ntile,
                                                              part.as<double>());
  pair_reduce_kernel<<<(npairs + 7) / 8, 256, 0, s>>>(part.as<double>(), ntp, pairs.as<int>(),
                                                     npairs, nocc, Epair);
  total_reduce_kernel<<<1, 1024, 0, s>>>(Epair, nocc, Etot);
  count_launch(4);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

// A planned plain FP64 batch: fragment table, per-item partials, queue.
struct PlainPlan {
  int nfrag = 0, npairs_total = 0, grid = 0;
  long long nitems = 0;
  std::vector<PlainFrag> fh;  // host copy of the descriptor table
  DevBuf frags, part, queue;
};

int plain_plan_create(PlainPlan **out, int nfrag, const PlainFrag *in, cudaStream_t s) {
  *out = nullptr;
  std::vector<PlainFrag> fh(in, in + nfrag);
  // heaviest items (longest K) first in the queue
  std::stable_sort(fh.begin(), fh.end(),
                   [](const PlainFrag &x, const PlainFrag &y) { return x.NBA > y.NBA; });
  long long item = 0;
  int pb = 0;
  for (auto &F : fh) {
    const int nt = (F.nvirt + TM - 1) / TM;
    F.ntp = nt * (nt + 1) / 2;
    F.pair_base = pb;
    F.item_base = item;
    const int np = F.nocc * (F.nocc + 1) / 2;
    pb += np;
    item += (long long)np * F.ntp;
  }
  if (item >= 2147483647LL) {
    set_error("plain batch too large for one launch (%lld items)", item);
    return RIMP2_ERR_ARG;
  }
  PlainPlan *P = new PlainPlan();
  P->nfrag = nfrag;
  P->npairs_total = pb;
  P->nitems = item;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, plain_batch_kernel, NTHR, 0);
  if (e != cudaSuccess || occ < 1) occ = 1;
  P->grid = (int)std::min<long long>(item > 0 ? item : 1, (long long)nsm * occ);
  int rc = P->frags.alloc(sizeof(PlainFrag) * (size_t)nfrag, s);
  if (rc == RIMP2_OK) rc = P->part.alloc(sizeof(double) * (size_t)std::max<long long>(item, 1), s);
  if (rc == RIMP2_OK) rc = P->queue.alloc(sizeof(unsigned int), s);
  P->fh = fh;
  if (rc == RIMP2_OK &&
      cudaMemcpyAsync(P->frags.p, P->fh.data(), sizeof(PlainFrag) * (size_t)nfrag,
                      cudaMemcpyHostToDevice, s) != cudaSuccess) {
    set_error("plain batch descriptor copy failed");
    rc = RIMP2_ERR_CUDA;
  }
  if (rc != RIMP2_OK) {
    delete P;
    return rc;
  }
  *out = P;
  return RIMP2_OK;
}

int plain_plan_launches(const PlainPlan *P) { return P && P->nfrag ? 3 : 0; }

int plain_plan_record(PlainPlan *P, cudaStream_t s) {
  if (!P || P->nfrag == 0) return RIMP2_OK;
  if (inject_fault("launch")) {
    set_error("injected launch failure (RIMP2_FAULT_INJECT=launch)");
    return RIMP2_ERR_CUDA;
  }
  const PlainFrag *fr = P->frags.as<PlainFrag>();
  RIMP2_CK(cudaMemsetAsync(P->queue.p, 0, sizeof(unsigned int), s));
  plain_batch_kernel<<<P->grid, NTHR, 0, s>>>(fr, P->nfrag, P->nitems, P->queue.as<unsigned int>(),
                                              P->part.as<double>());
  pair_reduce_plain_batch_kernel<<<(unsigned)((P->npairs_total + 7) / 8), 256, 0, s>>>(
      fr, P->nfrag, P->npairs_total, P->part.as<double>());
  total_reduce_plain_batch_kernel<<<P->nfrag, 1024, 0, s>>>(fr);
  count_launch(3);
  RIMP2_CK(cudaGetLastError());
  return RIMP2_OK;
}

void plain_plan_destroy(PlainPlan *P) { delete P; }

}  // namespace rimp2
