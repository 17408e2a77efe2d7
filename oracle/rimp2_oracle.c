/*
 * rimp2_oracle.c -- CPU oracle for the RI-MP2 amplitude / integral / energy path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; it is used by the tests, by the smoke check and by the
 * CPU-baseline leg of the benchmark, always as the checker (never as the
 * thing that is measured on the GPU path or shipped).
 *
 * What it restates (file:line of the reference project januseriksen/rimp2_gpu):
 *   - the nine CONTAINS subroutines of RIMP2.F90 (RIMP2.F90:381-641), each with
 *     the same loop nest and the same accumulation order inside one output
 *     element (the alpha loop runs 1..NBA sequentially, the projection loops
 *     run 1..n sequentially), so that results agree bit-for-bit with a
 *     serial Fortran build of the reference;
 *   - the Step 5-8 driver sequence of RIMP2.F90:71-170 (first_order=.false.)
 *     including its six column-major dgemm calls (RIMP2.F90:79,87,110,118,
 *     137,160), with a plain triple-loop dgemm in place of the vendor BLAS;
 *   - the constant-valued fixture generator of generate.F90:77-128 and the
 *     Fortran unformatted sequential record layout it writes
 *     (generate.F90:75-128,333-336; 4-byte record markers).
 *
 * What it adds (no counterpart in the reference, so parity of these parts is
 * pinned only by the identities in the tests, not by reference outputs):
 *   - closed-shell MP2 pair energies e_ij = sum_ab t_ij^ab (2 g_ij^ab - g_ij^ba)
 *     with t = g / (e_i + e_j - e_a - e_b), built from the same g as
 *     RIMP2_calc_toccA (RIMP2.F90:397-404), summed with Neumaier compensation;
 *   - Philox4x32-10 counter-based generator (Salmon et al., SC'11) with
 *     Box-Muller normals for the seeded synthetic inputs;
 *   - AO->MO three-centre transform, Cholesky factorisation of the auxiliary
 *     metric and the forward triangular solve that forms Calpha.
 *
 * All arrays are FP64, column-major, indexed exactly as the Fortran declares
 * them (first index fastest).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define I2(a, b, n1) ((size_t)(a) + (size_t)(n1) * (size_t)(b))
#define I3(a, b, c, n1, n2) ((size_t)(a) + (size_t)(n1) * ((size_t)(b) + (size_t)(n2) * (size_t)(c)))
#define I4(a, b, c, d, n1, n2, n3) \
  ((size_t)(a) + (size_t)(n1) * ((size_t)(b) + (size_t)(n2) * ((size_t)(c) + (size_t)(n3) * (size_t)(d))))

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* RIMP2_calc_toccA  (RIMP2.F90:381-417)                                    */
/* tocc(i,jL,a,b) = sum_j [sum_alpha C(alpha,a,i) C(alpha,b,j) / D] U(j,jL) */
/* ------------------------------------------------------------------------ */
void orc_calc_toccA(int nvirt, int nocc, int noccEOS, int NBA, const double *Calpha,
                    const double *EVocc, const double *EVvirt, double *tocc,
                    const double *UoccEOST) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int b = 0; b < nvirt; ++b)
    for (int a = 0; a < nvirt; ++a) {
      double tmpv[4096];
      double *toccTMP = nocc <= 4096 ? tmpv : (double *)malloc(sizeof(double) * nocc);
      for (int i = 0; i < nocc; ++i) {
        for (int j = 0; j < nocc; ++j) {
          double g = 0.0;
          const double *ca = Calpha + I3(0, a, i, NBA, nvirt);
          const double *cb = Calpha + I3(0, b, j, NBA, nvirt);
          for (int al = 0; al < NBA; ++al) g = g + ca[al] * cb[al]; /* RIMP2.F90:400-402 */
          double d = EVocc[i] + EVocc[j] - EVvirt[b] - EVvirt[a];   /* RIMP2.F90:403 */
          toccTMP[j] = g / d;                                       /* RIMP2.F90:404 */
        }
        for (int jl = 0; jl < noccEOS; ++jl) { /* RIMP2.F90:406-412 */
          double t = 0.0;
          for (int j = 0; j < nocc; ++j) t = t + toccTMP[j] * UoccEOST[I2(j, jl, nocc)];
          tocc[I4(i, jl, a, b, nocc, noccEOS, nvirt)] = t;
        }
      }
      if (toccTMP != tmpv) free(toccTMP);
    }
}

/* RIMP2_calc_tvirtA (RIMP2.F90:419-453) */
void orc_calc_tvirtA(int nvirt, int nocc, int nvirtEOS, int NBA, const double *Calpha,
                     const double *EVocc, const double *EVvirt, double *tvirt,
                     const double *UvirtEOST) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < nocc; ++j)
    for (int i = 0; i < nocc; ++i) {
      double *tvirtTMP = (double *)malloc(sizeof(double) * (size_t)nvirt);
      for (int b = 0; b < nvirt; ++b) {
        for (int a = 0; a < nvirt; ++a) {
          double g = 0.0;
          const double *ca = Calpha + I3(0, a, i, NBA, nvirt);
          const double *cb = Calpha + I3(0, b, j, NBA, nvirt);
          for (int al = 0; al < NBA; ++al) g = g + ca[al] * cb[al]; /* RIMP2.F90:436-438 */
          double d = EVocc[i] + EVocc[j] - EVvirt[b] - EVvirt[a];   /* RIMP2.F90:439 */
          tvirtTMP[a] = g / d;
        }
        for (int al = 0; al < nvirtEOS; ++al) { /* RIMP2.F90:442-448 */
          double t = 0.0;
          for (int a = 0; a < nvirt; ++a) t = t + tvirtTMP[a] * UvirtEOST[I2(a, al, nvirt)];
          tvirt[I4(i, j, al, b, nocc, nocc, nvirtEOS)] = t;
        }
      }
      free(tvirtTMP);
    }
}

/* RIMP2_calc_toccB (RIMP2.F90:456-481):
 * toccEOS(aL,iL,bL,jL) = sum_A tocc(iL,jL,A,bL) UvirtT(A,aL) */
void orc_calc_toccB(int nvirt, int noccEOS, const double *tocc, const double *UvirtT,
                    double *toccEOS) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int bl = 0; bl < nvirt; ++bl)
    for (int jl = 0; jl < noccEOS; ++jl)
      for (int al = 0; al < nvirt; ++al)
        for (int il = 0; il < noccEOS; ++il) {
          double t = 0.0;
          for (int A = 0; A < nvirt; ++A)
            t = t + tocc[I4(il, jl, A, bl, noccEOS, noccEOS, nvirt)] * UvirtT[I2(A, al, nvirt)];
          toccEOS[I4(al, il, bl, jl, nvirt, noccEOS, nvirt)] = t;
        }
}

/* RIMP2_calc_tvirtB (RIMP2.F90:483-508):
 * tvirtEOS(aL,iL,bL,jL) = sum_J tvirt(iL,J,aL,bL) UoccT(J,jL) */
void orc_calc_tvirtB(int nvirtEOS, int nocc, const double *tvirt, const double *UoccT,
                     double *tvirtEOS) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int jl = 0; jl < nocc; ++jl)
    for (int bl = 0; bl < nvirtEOS; ++bl)
      for (int il = 0; il < nocc; ++il)
        for (int al = 0; al < nvirtEOS; ++al) {
          double t = 0.0;
          for (int J = 0; J < nocc; ++J)
            t = t + tvirt[I4(il, J, al, bl, nocc, nocc, nvirtEOS)] * UoccT[I2(J, jl, nocc)];
          tvirtEOS[I4(al, il, bl, jl, nvirtEOS, nocc, nvirtEOS)] = t;
        }
}

/* RIMP2_TransAlpha1 (RIMP2.F90:510-533):
 * AlphaCD5(alpha,bL,jL) = sum_B UvirtT(B,bL) AlphaCD4(alpha,B,jL) */
void orc_transalpha1(int nvirt, int noccEOS, int nba, const double *UvirtT,
                     const double *AlphaCD4, double *AlphaCD5) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int jl = 0; jl < noccEOS; ++jl)
    for (int bl = 0; bl < nvirt; ++bl)
      for (int al = 0; al < nba; ++al) {
        double t = 0.0;
        for (int B = 0; B < nvirt; ++B)
          t = t + UvirtT[I2(B, bl, nvirt)] * AlphaCD4[I3(al, B, jl, nba, nvirt)];
        AlphaCD5[I3(al, bl, jl, nba, nvirt)] = t;
      }
}

/* RIMP2_TransAlpha2 (RIMP2.F90:536-560):
 * AlphaCD5(alpha,n3,n2) = sum_n1 U(n1,n3) AlphaCD4(alpha,n1,n2) */
void orc_transalpha2(int n2, int n1, int n3, int nba, const double *U, const double *AlphaCD4,
                     double *AlphaCD5) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int jl = 0; jl < n2; ++jl)
    for (int bl = 0; bl < n3; ++bl)
      for (int al = 0; al < nba; ++al) {
        double t = 0.0;
        for (int B = 0; B < n1; ++B) t = t + U[I2(B, bl, n1)] * AlphaCD4[I3(al, B, jl, nba, n1)];
        AlphaCD5[I3(al, bl, jl, nba, n3)] = t;
      }
}

/* Gram of a transformed three-centre array; shared loop body of
 * RIMP2_calc_gocc (RIMP2.F90:562-587), RIMP2_calc_gvirt (RIMP2.F90:589-614)
 * and RIMP2_calc_gen4DimFO (RIMP2.F90:616-641):
 * out(a,b,c,d) = sum_alpha X(alpha,a,b) Y(alpha,c,d) */
void orc_gen4dimfo(int NBA, const double *X, int n1, int n2, const double *Y, int n3, int n4,
                   double *out) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int d = 0; d < n4; ++d)
    for (int c = 0; c < n3; ++c)
      for (int b = 0; b < n2; ++b)
        for (int a = 0; a < n1; ++a) {
          double t = 0.0;
          const double *xa = X + I3(0, a, b, NBA, n1);
          const double *yc = Y + I3(0, c, d, NBA, n3);
          for (int al = 0; al < NBA; ++al) t = t + xa[al] * yc[al];
          out[I4(a, b, c, d, n1, n2, n3)] = t;
        }
}

void orc_calc_gocc(int nvirt, int noccEOS, int NBA, const double *Calpha3, double *goccEOS) {
  orc_gen4dimfo(NBA, Calpha3, nvirt, noccEOS, Calpha3, nvirt, noccEOS, goccEOS);
}

void orc_calc_gvirt(int nvirtEOS, int nocc, int NBA, const double *Calpha3, double *gvirtEOS) {
  orc_gen4dimfo(NBA, Calpha3, nvirtEOS, nocc, Calpha3, nvirtEOS, nocc, gvirtEOS);
}

/* Column-major dgemm with reference-BLAS semantics:
 * C = alpha*op(A)*op(B) + beta*C, the k sum running 0..K-1 in order. */
void orc_dgemm(char ta, char tb, int M, int N, int K, double alpha, const double *A, int lda,
               const double *B, int ldb, double beta, double *C, int ldc) {
  int tA = (ta == 'T' || ta == 't'), tB = (tb == 'T' || tb == 't');
#pragma omp parallel for collapse(2) schedule(static)
  for (int n = 0; n < N; ++n)
    for (int m = 0; m < M; ++m) {
      double s = 0.0;
      for (int k = 0; k < K; ++k) {
        double av = tA ? A[I2(k, m, lda)] : A[I2(m, k, lda)];
        double bv = tB ? B[I2(n, k, ldb)] : B[I2(k, n, ldb)];
        s += av * bv;
      }
      double c = (beta == 0.0) ? 0.0 : beta * C[I2(m, n, ldc)];
      C[I2(m, n, ldc)] = alpha * s + c;
    }
}

/* ------------------------------------------------------------------------ */
/* Steps 5-8 of the driver (RIMP2.F90:71-170, first_order = .false.)        */
/* ------------------------------------------------------------------------ */
int orc_steps5to8(int nvirt, int nocc, int noccEOS, int nvirtEOS, int NBA, const double *Calpha,
                  const double *EVocc, const double *EVvirt, const double *UoccEOST,
                  const double *UvirtT, const double *UoccT, const double *UvirtEOST,
                  double *toccEOS, double *tvirtEOS, double *goccEOS, double *gvirtEOS) {
  size_t nv = nvirt, no = nocc, noE = noccEOS, nvE = nvirtEOS, nb = NBA;
  /* Step 5 (RIMP2.F90:71-93) */
  double *tocc = (double *)malloc(sizeof(double) * no * noE * nv * nv);
  double *tocc2 = (double *)malloc(sizeof(double) * noE * noE * nv * nv);
  double *tocc3 = (double *)malloc(sizeof(double) * nv * nv * noE * noE);
  if (!tocc || !tocc2 || !tocc3) return 1;
  orc_calc_toccA(nvirt, nocc, noccEOS, NBA, Calpha, EVocc, EVvirt, tocc, UoccEOST);
  orc_dgemm('T', 'N', noccEOS, noccEOS * nvirt * nvirt, nocc, 1.0, UoccEOST, nocc, tocc, nocc, 0.0,
            tocc2, noccEOS);
  orc_dgemm('N', 'N', noccEOS * noccEOS * nvirt, nvirt, nvirt, 1.0, tocc2, noccEOS * noccEOS * nvirt,
            UvirtT, nvirt, 0.0, tocc3, noccEOS * noccEOS * nvirt);
  orc_calc_toccB(nvirt, noccEOS, tocc3, UvirtT, toccEOS);
  free(tocc);
  free(tocc2);
  free(tocc3);
  /* Step 6 (RIMP2.F90:99-124) */
  double *tvirt = (double *)malloc(sizeof(double) * no * no * nvE * nv);
  double *tvirt2 = (double *)malloc(sizeof(double) * no * no * nvE * nvE);
  double *tvirt3 = (double *)malloc(sizeof(double) * no * no * nvE * nvE);
  if (!tvirt || !tvirt2 || !tvirt3) return 1;
  orc_calc_tvirtA(nvirt, nocc, nvirtEOS, NBA, Calpha, EVocc, EVvirt, tvirt, UvirtEOST);
  orc_dgemm('N', 'N', nocc * nocc * nvirtEOS, nvirtEOS, nvirt, 1.0, tvirt, nocc * nocc * nvirtEOS,
            UvirtEOST, nvirt, 0.0, tvirt2, nocc * nocc * nvirtEOS);
  orc_dgemm('T', 'N', nocc, nocc * nvirtEOS * nvirtEOS, nocc, 1.0, UoccT, nocc, tvirt2, nocc, 0.0,
            tvirt3, nocc);
  orc_calc_tvirtB(nvirtEOS, nocc, tvirt3, UoccT, tvirtEOS);
  free(tvirt);
  free(tvirt2);
  free(tvirt3);
  /* Step 7 (RIMP2.F90:133-147) */
  double *C2 = (double *)malloc(sizeof(double) * nb * nv * (no > nvE ? no : nvE));
  double *C3 = (double *)malloc(sizeof(double) * nb * nv * (no > nvE ? no : nvE));
  if (!C2 || !C3) return 1;
  orc_dgemm('N', 'N', NBA * nvirt, noccEOS, nocc, 1.0, Calpha, NBA * nvirt, UoccEOST, nocc, 0.0, C2,
            NBA * nvirt);
  orc_transalpha1(nvirt, noccEOS, NBA, UvirtT, C2, C3);
  orc_calc_gocc(nvirt, noccEOS, NBA, C3, goccEOS);
  /* Step 8 (RIMP2.F90:155-170) */
  orc_dgemm('N', 'N', NBA * nvirt, nocc, nocc, 1.0, Calpha, NBA * nvirt, UoccT, nocc, 0.0, C2,
            NBA * nvirt);
  orc_transalpha2(nocc, nvirt, nvirtEOS, NBA, UvirtEOST, C2, C3);
  orc_calc_gvirt(nvirtEOS, nocc, NBA, C3, gvirtEOS);
  free(C2);
  free(C3);
  return 0;
}

/* First-order property integrals of the driver (RIMP2.F90:172-251, run when
 * first_order = .TRUE., RIMP2.F90:65; same sequence in generate.F90:237-331).
 * djik(nvirt,noccEOS,noccEOS,nocctot), blad(nvirtEOS,nocc,nvirtEOS,nvirt).
 * UoccallT is the (nocctot,nocctot) matrix the djik DGEMM reads
 * (RIMP2.F90:192-197 passes UoccT there, which is the same array when
 * nocctot = nocc).  The CalphaVV DGEMM keeps the driver's K = ldb = nocc
 * (RIMP2.F90:232-235). */
int orc_first_order(int nvirt, int nocc, int noccEOS, int nvirtEOS, int nocctot, int NBA,
                    const double *Calpha, const double *CalphaOcc, const double *CalphaVV,
                    const double *UoccEOST, const double *UvirtT, const double *UoccT,
                    const double *UoccallT, const double *UvirtEOST, double *djik, double *blad) {
  size_t nv = nvirt, no = nocc, noE = noccEOS, nvE = nvirtEOS, nb = NBA, nt = nocctot;
  size_t big = nb * nv * (nv > no ? nv : no);
  if (nb * no * nt > big) big = nb * no * nt;
  double *C2 = (double *)malloc(sizeof(double) * big);
  double *C3 = (double *)malloc(sizeof(double) * big);
  double *C4 = (double *)malloc(sizeof(double) * big);
  if (!C2 || !C3 || !C4) return 1;
  /* djik: RIMP2.F90:177-207 */
  orc_dgemm('N', 'N', NBA * nvirt, noccEOS, nocc, 1.0, Calpha, NBA * nvirt, UoccEOST, nocc, 0.0, C2,
            NBA * nvirt);                                            /* :177-182 */
  orc_transalpha2(noccEOS, nvirt, nvirt, NBA, UvirtT, C2, C3);      /* :186 */
  orc_dgemm('N', 'N', NBA * nocc, nocctot, nocctot, 1.0, CalphaOcc, NBA * nocc, UoccallT, nocctot,
            0.0, C2, NBA * nocc);                                    /* :192-197 */
  orc_transalpha2(nocctot, nocc, noccEOS, NBA, UoccEOST, C2, C4);   /* :201 */
  orc_gen4dimfo(NBA, C3, nvirt, noccEOS, C4, noccEOS, nocctot, djik); /* :207 */
  /* blad: RIMP2.F90:216-248 */
  orc_dgemm('N', 'N', NBA * nvirt, nocc, nocc, 1.0, Calpha, NBA * nvirt, UoccT, nocc, 0.0, C2,
            NBA * nvirt);                                            /* :216-220 */
  orc_transalpha2(nocc, nvirt, nvirtEOS, NBA, UvirtEOST, C2, C3);   /* :225 */
  orc_dgemm('N', 'N', NBA * nvirt, nvirt, nocc, 1.0, CalphaVV, NBA * nvirt, UvirtT, nocc, 0.0, C2,
            NBA * nvirt);                                            /* :232-235 */
  orc_transalpha2(nvirt, nvirt, nvirtEOS, NBA, UvirtEOST, C2, C4);  /* :242 */
  orc_gen4dimfo(NBA, C3, nvirtEOS, nocc, C4, nvirtEOS, nvirt, blad); /* :248 */
  free(C2);
  free(C3);
  free(C4);
  (void)noE;
  (void)nvE;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* MP2 pair energies (restated; no counterpart in the reference)            */
/* ------------------------------------------------------------------------ */
static inline void neumaier_add(double *s, double *c, double x) {
  double t = *s + x;
  if (fabs(*s) >= fabs(x))
    *c += (*s - t) + x;
  else
    *c += (x - t) + *s;
  *s = t;
}

/* Faithful form: g_ij(a,b) and g_ij(b,a) each built with the sequential alpha
 * loop of RIMP2.F90:400-402 and the denominator of RIMP2.F90:403.
 * pairs: npairs (i,j) index pairs (0-based, interleaved), or NULL for all
 * i<=j.  Epair is nocc x nocc column-major; both (i,j) and (j,i) are written.
 * Returns the compensated total over all requested pairs counted with their
 * multiplicity in the full double sum over (i,j). */
double orc_pair_energies(int nvirt, int nocc, int NBA, const double *Calpha, const double *EVocc,
                         const double *EVvirt, double *Epair, const int *pairs, int npairs) {
  int np = pairs ? npairs : nocc * (nocc + 1) / 2;
  int *pl = (int *)malloc(sizeof(int) * 2 * (size_t)np);
  if (pairs)
    memcpy(pl, pairs, sizeof(int) * 2 * (size_t)np);
  else {
    int k = 0;
    for (int j = 0; j < nocc; ++j)
      for (int i = 0; i <= j; ++i) {
        pl[2 * k] = i;
        pl[2 * k + 1] = j;
        ++k;
      }
  }
  double *ep = (double *)malloc(sizeof(double) * (size_t)np);
  /* one task per (pair, b): the b-loop of RIMP2.F90:395 is the parallel one,
   * as in the reference's COLLAPSE over (BDIAG,ADIAG) */
  double *part = (double *)malloc(sizeof(double) * (size_t)np * nvirt);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long task = 0; task < (long long)np * nvirt; ++task) {
    int p = (int)(task / nvirt), b = (int)(task % nvirt);
    int i = pl[2 * p], j = pl[2 * p + 1];
    double s = 0.0, c = 0.0;
    for (int a = 0; a < nvirt; ++a) {
      const double *cai = Calpha + I3(0, a, i, NBA, nvirt);
      const double *cbj = Calpha + I3(0, b, j, NBA, nvirt);
      const double *cbi = Calpha + I3(0, b, i, NBA, nvirt);
      const double *caj = Calpha + I3(0, a, j, NBA, nvirt);
      double g = 0.0, gx = 0.0;
      for (int al = 0; al < NBA; ++al) g = g + cai[al] * cbj[al];   /* RIMP2.F90:400-402 */
      for (int al = 0; al < NBA; ++al) gx = gx + cbi[al] * caj[al];
      double d = EVocc[i] + EVocc[j] - EVvirt[b] - EVvirt[a];       /* RIMP2.F90:403 */
      neumaier_add(&s, &c, (g / d) * (2.0 * g - gx));
    }
    part[task] = s + c;
  }
  for (int p = 0; p < np; ++p) {
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nvirt; ++b) neumaier_add(&s, &c, part[(size_t)p * nvirt + b]);
    ep[p] = s + c;
  }
  free(part);
  double ts = 0.0, tc = 0.0;
  for (int p = 0; p < np; ++p) {
    int i = pl[2 * p], j = pl[2 * p + 1];
    if (Epair) {
      Epair[I2(i, j, nocc)] = ep[p];
      Epair[I2(j, i, nocc)] = ep[p];
    }
    neumaier_add(&ts, &tc, ep[p]);
    if (i != j) neumaier_add(&ts, &tc, ep[p]);
  }
  free(pl);
  free(ep);
  return ts + tc;
}

/* Cache-blocked form of the same energy (identical formula, FP64 throughout,
 * four interleaved partial sums per dot product).  Used where the faithful
 * loop order would take too long; agrees with orc_pair_energies to ~1e-15
 * relative. */
double orc_pair_energies_blocked(int nvirt, int nocc, int NBA, const double *Calpha,
                                 const double *EVocc, const double *EVvirt, double *Epair,
                                 const int *pairs, int npairs) {
  int np = pairs ? npairs : nocc * (nocc + 1) / 2;
  int *pl = (int *)malloc(sizeof(int) * 2 * (size_t)np);
  if (pairs)
    memcpy(pl, pairs, sizeof(int) * 2 * (size_t)np);
  else {
    int k = 0;
    for (int j = 0; j < nocc; ++j)
      for (int i = 0; i <= j; ++i) {
        pl[2 * k] = i;
        pl[2 * k + 1] = j;
        ++k;
      }
  }
  const int BT = 16;
  int nbt = (nvirt + BT - 1) / BT;
  int ntask = np * nbt * nbt;
  double *part = (double *)calloc((size_t)ntask, sizeof(double));
#pragma omp parallel for schedule(dynamic, 1)
  for (int task = 0; task < ntask; ++task) {
    int p = task / (nbt * nbt), r = task % (nbt * nbt);
    int ab = r % nbt, bb = r / nbt;
    int i = pl[2 * p], j = pl[2 * p + 1];
    double s = 0.0, c = 0.0;
    for (int b = bb * BT; b < nvirt && b < (bb + 1) * BT; ++b)
      for (int a = ab * BT; a < nvirt && a < (ab + 1) * BT; ++a) {
        const double *cai = Calpha + I3(0, a, i, NBA, nvirt);
        const double *cbj = Calpha + I3(0, b, j, NBA, nvirt);
        const double *cbi = Calpha + I3(0, b, i, NBA, nvirt);
        const double *caj = Calpha + I3(0, a, j, NBA, nvirt);
        double g0 = 0, g1 = 0, g2 = 0, g3 = 0, x0 = 0, x1 = 0, x2 = 0, x3 = 0;
        int al = 0;
        for (; al + 4 <= NBA; al += 4) {
          g0 += cai[al] * cbj[al];
          g1 += cai[al + 1] * cbj[al + 1];
          g2 += cai[al + 2] * cbj[al + 2];
          g3 += cai[al + 3] * cbj[al + 3];
          x0 += cbi[al] * caj[al];
          x1 += cbi[al + 1] * caj[al + 1];
          x2 += cbi[al + 2] * caj[al + 2];
          x3 += cbi[al + 3] * caj[al + 3];
        }
        for (; al < NBA; ++al) {
          g0 += cai[al] * cbj[al];
          x0 += cbi[al] * caj[al];
        }
        double g = (g0 + g1) + (g2 + g3), gx = (x0 + x1) + (x2 + x3);
        double d = EVocc[i] + EVocc[j] - EVvirt[b] - EVvirt[a];
        neumaier_add(&s, &c, (g / d) * (2.0 * g - gx));
      }
    part[task] = s + c;
  }
  double ts = 0.0, tc = 0.0;
  for (int p = 0; p < np; ++p) {
    double s = 0.0, c = 0.0;
    for (int r = 0; r < nbt * nbt; ++r) neumaier_add(&s, &c, part[(size_t)p * nbt * nbt + r]);
    double e = s + c;
    int i = pl[2 * p], j = pl[2 * p + 1];
    if (Epair) {
      Epair[I2(i, j, nocc)] = e;
      Epair[I2(j, i, nocc)] = e;
    }
    neumaier_add(&ts, &tc, e);
    if (i != j) neumaier_add(&ts, &tc, e);
  }
  free(part);
  free(pl);
  return ts + tc;
}

/* Canonical amplitudes t(a,i,b,j) = g_ij(a,b)/D, layout (nvirt,nocc,nvirt,nocc)
 * -- the toccEOS layout of RIMP2.F90:91 when U = I. */
void orc_amplitudes(int nvirt, int nocc, int NBA, const double *Calpha, const double *EVocc,
                    const double *EVvirt, double *t) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int j = 0; j < nocc; ++j)
    for (int b = 0; b < nvirt; ++b)
      for (int i = 0; i < nocc; ++i)
        for (int a = 0; a < nvirt; ++a) {
          const double *cai = Calpha + I3(0, a, i, NBA, nvirt);
          const double *cbj = Calpha + I3(0, b, j, NBA, nvirt);
          double g = 0.0;
          for (int al = 0; al < NBA; ++al) g = g + cai[al] * cbj[al];
          double d = EVocc[i] + EVocc[j] - EVvirt[b] - EVvirt[a];
          t[I4(a, i, b, j, nvirt, nocc, nvirt)] = g / d;
        }
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) + Box-Muller            */
/* ------------------------------------------------------------------------ */
static inline uint32_t mulhilo32(uint32_t a, uint32_t b, uint32_t *hi) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  return (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, hi1;
    uint32_t lo0 = mulhilo32(0xD2511F53u, c0, &hi0);
    uint32_t lo1 = mulhilo32(0xCD9E8D57u, c2, &hi1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* two uniforms in (0,1) with 53-bit resolution from counter (n, stream) */
static inline void philox_u2(uint64_t seed, uint32_t stream, uint64_t n, double *u0, double *u1) {
  uint32_t ctr[4] = {(uint32_t)n, (uint32_t)(n >> 32), stream, 0x5249u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  uint64_t a = ((uint64_t)(o[0] >> 5) << 26) | (uint64_t)(o[1] >> 6);
  uint64_t b = ((uint64_t)(o[2] >> 5) << 26) | (uint64_t)(o[3] >> 6);
  *u0 = ((double)a + 0.5) * (1.0 / 9007199254740992.0);
  *u1 = ((double)b + 0.5) * (1.0 / 9007199254740992.0);
}

/* n-th standard normal of stream `stream` (Box-Muller on uniform pair n/2) */
static inline double philox_normal(uint64_t seed, uint32_t stream, uint64_t n) {
  double u0, u1;
  philox_u2(seed, stream, n >> 1, &u0, &u1);
  double r = sqrt(-2.0 * log(u0));
  double th = 6.283185307179586476925286766559 * u1;
  return (n & 1) ? r * sin(th) : r * cos(th);
}

double orc_uniform(uint64_t seed, uint32_t stream, uint64_t n) {
  double u0, u1;
  philox_u2(seed, stream, n >> 1, &u0, &u1);
  return (n & 1) ? u1 : u0;
}

double orc_normal(uint64_t seed, uint32_t stream, uint64_t n) { return philox_normal(seed, stream, n); }

/* Calpha(alpha,a,i) = N(0,1) * 0.03 / sqrt(1 + alpha/64), alpha 0-based,
 * normal number = column-major linear index of the element in stream 0. */
void orc_gen_calpha(uint64_t seed, int NBA, int nvirt, int nocc, double *Calpha) {
  size_t tot = (size_t)NBA * nvirt * nocc;
#pragma omp parallel for schedule(static)
  for (size_t n = 0; n < tot; n += 2) {
    double u0, u1;
    philox_u2(seed, 0u, n >> 1, &u0, &u1);
    double r = sqrt(-2.0 * log(u0));
    double th = 6.283185307179586476925286766559 * u1;
    int al0 = (int)(n % (size_t)NBA);
    Calpha[n] = r * cos(th) * 0.03 / sqrt(1.0 + al0 / 64.0);
    if (n + 1 < tot) {
      int al1 = (int)((n + 1) % (size_t)NBA);
      Calpha[n + 1] = r * sin(th) * 0.03 / sqrt(1.0 + al1 / 64.0);
    }
  }
}

/* Calpha(:,:,occ[k]) of the full fragment (nocc occupied) for a subset of
 * occupied indices, written as out(NBA,nvirt,nsel): the same numbers
 * orc_gen_calpha would put there. */
void orc_gen_calpha_slabs(uint64_t seed, int NBA, int nvirt, const int *occ, int nsel, double *out) {
  size_t slab = (size_t)NBA * nvirt;
#pragma omp parallel for schedule(static)
  for (long long t = 0; t < (long long)nsel * (long long)slab; ++t) {
    int k = (int)(t / (long long)slab);
    size_t r = (size_t)(t % (long long)slab);
    size_t n = (size_t)occ[k] * slab + r;
    int al = (int)(n % (size_t)NBA);
    out[t] = philox_normal(seed, 0u, n) * 0.03 / sqrt(1.0 + al / 64.0);
  }
}

static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

/* eps_occ sorted U[-1.5,-0.3] (stream 1), eps_virt sorted U[0.1,3.0] (stream 2) */
void orc_gen_eps(uint64_t seed, int nocc, int nvirt, double *EVocc, double *EVvirt) {
  for (int i = 0; i < nocc; ++i) EVocc[i] = -1.5 + 1.2 * orc_uniform(seed, 1u, (uint64_t)i);
  for (int a = 0; a < nvirt; ++a) EVvirt[a] = 0.1 + 2.9 * orc_uniform(seed, 2u, (uint64_t)a);
  qsort(EVocc, (size_t)nocc, sizeof(double), cmp_double);
  qsort(EVvirt, (size_t)nvirt, sizeof(double), cmp_double);
}

/* general (non-orthogonal) rotation matrix, N(0,1)/sqrt(n1), stream s */
void orc_gen_matrix(uint64_t seed, uint32_t stream, int n1, int n2, double *U) {
  double sc = 1.0 / sqrt((double)n1);
  for (size_t n = 0; n < (size_t)n1 * n2; ++n) U[n] = philox_normal(seed, stream, n) * sc;
}

/* Constant-valued fixtures of generate.F90:77-128 (the reference's own
 * known-answer inputs): every element is a closed-form constant. */
void orc_gen_kat(int NBA, int nvirt, int nocc, int noccEOS, int nvirtEOS, double *Calpha,
                 double *EVocc, double *EVvirt, double *UoccEOST, double *UvirtT, double *UoccT,
                 double *UvirtEOST) {
  for (int c = 1; c <= nocc; ++c)
    for (int b = 1; b <= nvirt; ++b)
      for (int a = 1; a <= NBA; ++a)
        Calpha[I3(a - 1, b - 1, c - 1, NBA, nvirt)] =
            a * 0.00124235636 / a + b * 0.01010101 / b + c * 0.014321 / c; /* generate.F90:81 */
  for (int c = 1; c <= nocc; ++c) EVocc[c - 1] = c * 1.934321 / c;        /* :88 */
  for (int c = 1; c <= nvirt; ++c) EVvirt[c - 1] = c * 1.91321 / c;       /* :94 */
  for (int b = 1; b <= noccEOS; ++b)
    for (int a = 1; a <= nocc; ++a)
      UoccEOST[I2(a - 1, b - 1, nocc)] = a * 0.030321 / a + b * 0.101121 / b; /* :101 */
  for (int b = 1; b <= nvirt; ++b)
    for (int a = 1; a <= nvirt; ++a)
      UvirtT[I2(a - 1, b - 1, nvirt)] = a * 0.021321 / a + b * 0.01321 / b; /* :109 */
  for (int b = 1; b <= nocc; ++b)
    for (int a = 1; a <= nocc; ++a)
      UoccT[I2(a - 1, b - 1, nocc)] = a * 0.032321 / a + b * 0.01521 / b; /* :117 */
  for (int b = 1; b <= nvirtEOS; ++b)
    for (int a = 1; a <= nvirt; ++a)
      UvirtEOST[I2(a - 1, b - 1, nvirt)] = a * 0.023321 / a + b * 0.01421 / b; /* :125 */
}

/* First-order fixture inputs of generate.F90:254-260 (CalphaOcc) and
 * :300-306 (CalphaVV): A*0.01124235636 + B*0.01011111 + C*0.16422. */
void orc_gen_kat_fo(int NBA, int nvirt, int nocc, int nocctot, double *CalphaOcc,
                    double *CalphaVV) {
  for (int c = 1; c <= nocctot; ++c)
    for (int b = 1; b <= nocc; ++b)
      for (int a = 1; a <= NBA; ++a)
        CalphaOcc[I3(a - 1, b - 1, c - 1, NBA, nocc)] = a * 0.01124235636 + b * 0.01011111 + c * 0.16422;
  for (int c = 1; c <= nvirt; ++c)
    for (int b = 1; b <= nvirt; ++b)
      for (int a = 1; a <= NBA; ++a)
        CalphaVV[I3(a - 1, b - 1, c - 1, NBA, nvirt)] = a * 0.01124235636 + b * 0.01011111 + c * 0.16422;
}

/* ------------------------------------------------------------------------ */
/* Fortran unformatted sequential records (4-byte head/tail length markers) */
/* ------------------------------------------------------------------------ */
int orc_write_record(FILE *f, const void *data, size_t nbytes) {
  if (nbytes > 0x7fffffffu) return 1;
  int32_t m = (int32_t)nbytes;
  if (fwrite(&m, 4, 1, f) != 1) return 1;
  if (nbytes && fwrite(data, 1, nbytes, f) != nbytes) return 1;
  if (fwrite(&m, 4, 1, f) != 1) return 1;
  return 0;
}

int orc_read_record(FILE *f, void *data, size_t nbytes) {
  int32_t m0, m1;
  if (fread(&m0, 4, 1, f) != 1) return 1;
  if ((size_t)m0 != nbytes) return 2;
  if (nbytes && fread(data, 1, nbytes, f) != nbytes) return 1;
  if (fread(&m1, 4, 1, f) != 1) return 1;
  return m0 == m1 ? 0 : 3;
}

/* Write a Calpha{1,2}.data-style file: header record of six default integers,
 * then Calpha, EVocc, EVvirt, UoccEOST, UvirtT, UoccT, UvirtEOST, then the
 * golden toccEOS, tvirtEOS, gvirtEOS, goccEOS (generate.F90:75-128,333-336). */
int orc_write_datafile(const char *path, int nvirt, int nocc, int noccEOS, int nvirtEOS, int NBA,
                       int nocctot, const double *Calpha, const double *EVocc, const double *EVvirt,
                       const double *UoccEOST, const double *UvirtT, const double *UoccT,
                       const double *UvirtEOST, const double *toccEOS, const double *tvirtEOS,
                       const double *gvirtEOS, const double *goccEOS) {
  FILE *f = fopen(path, "wb");
  if (!f) return 1;
  int32_t hdr[6] = {nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot};
  size_t nv = nvirt, no = nocc, noE = noccEOS, nvE = nvirtEOS, nb = NBA;
  int rc = 0;
  rc |= orc_write_record(f, hdr, sizeof hdr);
  rc |= orc_write_record(f, Calpha, 8 * nb * nv * no);
  rc |= orc_write_record(f, EVocc, 8 * no);
  rc |= orc_write_record(f, EVvirt, 8 * nv);
  rc |= orc_write_record(f, UoccEOST, 8 * no * noE);
  rc |= orc_write_record(f, UvirtT, 8 * nv * nv);
  rc |= orc_write_record(f, UoccT, 8 * no * no);
  rc |= orc_write_record(f, UvirtEOST, 8 * nv * nvE);
  rc |= orc_write_record(f, toccEOS, 8 * nv * noE * nv * noE);
  rc |= orc_write_record(f, tvirtEOS, 8 * nvE * no * nvE * no);
  rc |= orc_write_record(f, gvirtEOS, 8 * nvE * no * nvE * no);
  rc |= orc_write_record(f, goccEOS, 8 * nv * noE * nv * noE);
  fclose(f);
  return rc;
}

/* Read the header record (RIMP2.F90:45) */
int orc_read_header(const char *path, int32_t hdr[6]) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  int rc = orc_read_record(f, hdr, 24);
  fclose(f);
  return rc;
}

/* Read every record after the header (RIMP2.F90:48-63 and :257,275,293,311) */
int orc_read_datafile(const char *path, double *Calpha, double *EVocc, double *EVvirt,
                      double *UoccEOST, double *UvirtT, double *UoccT, double *UvirtEOST,
                      double *toccEOS, double *tvirtEOS, double *gvirtEOS, double *goccEOS) {
  FILE *f = fopen(path, "rb");
  if (!f) return 1;
  int32_t h[6];
  int rc = orc_read_record(f, h, 24);
  if (rc) {
    fclose(f);
    return rc;
  }
  size_t nv = h[0], no = h[1], noE = h[2], nvE = h[3], nb = h[4];
  rc |= orc_read_record(f, Calpha, 8 * nb * nv * no);
  rc |= orc_read_record(f, EVocc, 8 * no);
  rc |= orc_read_record(f, EVvirt, 8 * nv);
  rc |= orc_read_record(f, UoccEOST, 8 * no * noE);
  rc |= orc_read_record(f, UvirtT, 8 * nv * nv);
  rc |= orc_read_record(f, UoccT, 8 * no * no);
  rc |= orc_read_record(f, UvirtEOST, 8 * nv * nvE);
  rc |= orc_read_record(f, toccEOS, 8 * nv * noE * nv * noE);
  rc |= orc_read_record(f, tvirtEOS, 8 * nvE * no * nvE * no);
  rc |= orc_read_record(f, gvirtEOS, 8 * nvE * no * nvE * no);
  rc |= orc_read_record(f, goccEOS, 8 * nv * noE * nv * noE);
  fclose(f);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Front end from AO three-centre integrals (restated; not in the reference) */
/* ------------------------------------------------------------------------ */
/* (alpha|mu nu) = N(0,1) exp(-|mu-nu|/32), symmetric in mu,nu; layout
 * ao(alpha, mu, nu) with alpha fastest.  Normal number = alpha + NBA*tri(mu,nu)
 * where tri is the packed index of mu<=nu; stream 3. */
void orc_gen_ao3c(uint64_t seed, int NBA, int nbas, double *ao) {
#pragma omp parallel for schedule(static)
  for (int nu = 0; nu < nbas; ++nu)
    for (int mu = 0; mu <= nu; ++mu) {
      size_t tri = (size_t)nu * (nu + 1) / 2 + mu;
      double w = exp(-fabs((double)(mu - nu)) / 32.0);
      for (int al = 0; al < NBA; ++al) {
        double v = philox_normal(seed, 3u, (size_t)al + (size_t)NBA * tri) * w;
        ao[I3(al, mu, nu, NBA, nbas)] = v;
        ao[I3(al, nu, mu, NBA, nbas)] = v;
      }
    }
}

/* V = A A^T / NBA + 0.1 I, A ~ N(0,1) (stream 4); V column-major NBA x NBA */
void orc_gen_metric(uint64_t seed, int NBA, double *V) {
  double *A = (double *)malloc(sizeof(double) * (size_t)NBA * NBA);
  for (size_t n = 0; n < (size_t)NBA * NBA; ++n) A[n] = philox_normal(seed, 4u, n);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < NBA; ++c)
    for (int r = 0; r < NBA; ++r) {
      double s = 0.0;
      for (int k = 0; k < NBA; ++k) s += A[I2(r, k, NBA)] * A[I2(c, k, NBA)];
      V[I2(r, c, NBA)] = s / NBA + (r == c ? 0.1 : 0.0);
    }
  free(A);
}

/* MO coefficients: Q of a Householder QR of a Gaussian nbas x nbas matrix
 * (stream 5), with column signs fixed so that diag(R) > 0.  Columns 0..nocc-1
 * are occupied, the rest virtual. */
void orc_gen_mo(uint64_t seed, int nbas, double *Cmo) {
  int n = nbas;
  double *A = (double *)malloc(sizeof(double) * (size_t)n * n);
  double *tau = (double *)malloc(sizeof(double) * (size_t)n);
  for (size_t k = 0; k < (size_t)n * n; ++k) A[k] = philox_normal(seed, 5u, k);
  for (int k = 0; k < n; ++k) {
    double nrm = 0.0;
    for (int r = k; r < n; ++r) nrm += A[I2(r, k, n)] * A[I2(r, k, n)];
    nrm = sqrt(nrm);
    double alpha = A[I2(k, k, n)] > 0 ? -nrm : nrm;
    double v0 = A[I2(k, k, n)] - alpha;
    double vn = v0 * v0;
    for (int r = k + 1; r < n; ++r) vn += A[I2(r, k, n)] * A[I2(r, k, n)];
    A[I2(k, k, n)] = v0;
    tau[k] = vn > 0 ? 2.0 / vn : 0.0;
    for (int c = k + 1; c < n; ++c) {
      double s = 0.0;
      for (int r = k; r < n; ++r) s += A[I2(r, k, n)] * A[I2(r, c, n)];
      s *= tau[k];
      for (int r = k; r < n; ++r) A[I2(r, c, n)] -= s * A[I2(r, k, n)];
    }
    A[I2(k, k, n)] = v0;
    /* store R diagonal sign in tau's companion: alpha */
    Cmo[I2(k, k, n)] = alpha; /* temporary */
  }
  double *sg = (double *)malloc(sizeof(double) * (size_t)n);
  for (int k = 0; k < n; ++k) sg[k] = Cmo[I2(k, k, n)] < 0 ? -1.0 : 1.0;
  /* Q = H_0 H_1 ... H_{n-1} applied to I */
  for (size_t k = 0; k < (size_t)n * n; ++k) Cmo[k] = 0.0;
  for (int k = 0; k < n; ++k) Cmo[I2(k, k, n)] = 1.0;
  for (int k = n - 1; k >= 0; --k)
    for (int c = 0; c < n; ++c) {
      double s = 0.0;
      for (int r = k; r < n; ++r) s += A[I2(r, k, n)] * Cmo[I2(r, c, n)];
      s *= tau[k];
      for (int r = k; r < n; ++r) Cmo[I2(r, c, n)] -= s * A[I2(r, k, n)];
    }
  for (int c = 0; c < n; ++c)
    for (int r = 0; r < n; ++r) Cmo[I2(r, c, n)] *= sg[c];
  free(sg);
  free(A);
  free(tau);
}

/* (alpha|a i) = sum_{mu,nu} Cv(mu,a) Co(nu,i) (alpha|mu nu); output in the
 * Calpha layout (alpha, a, i).  Cmo columns: 0..nocc-1 occ, nocc.. virt. */
void orc_ao2mo(int NBA, int nbas, int nocc, int nvirt, const double *ao, const double *Cmo,
               double *out) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nocc; ++i) {
    double *half = (double *)malloc(sizeof(double) * (size_t)NBA * nbas);
    /* half(alpha, mu) = sum_nu ao(alpha, mu, nu) Co(nu, i) */
    for (size_t k = 0; k < (size_t)NBA * nbas; ++k) half[k] = 0.0;
    for (int nu = 0; nu < nbas; ++nu) {
      double c = Cmo[I2(nu, i, nbas)];
      for (int mu = 0; mu < nbas; ++mu) {
        const double *src = ao + I3(0, mu, nu, NBA, nbas);
        double *dst = half + I2(0, mu, NBA);
        for (int al = 0; al < NBA; ++al) dst[al] += src[al] * c;
      }
    }
    for (int a = 0; a < nvirt; ++a) {
      double *dst = out + I3(0, a, i, NBA, nvirt);
      for (int al = 0; al < NBA; ++al) dst[al] = 0.0;
      for (int mu = 0; mu < nbas; ++mu) {
        double c = Cmo[I2(mu, nocc + a, nbas)];
        const double *src = half + I2(0, mu, NBA);
        for (int al = 0; al < NBA; ++al) dst[al] += src[al] * c;
      }
    }
    free(half);
  }
}

/* In-place lower Cholesky V = L L^T (column-major, lower triangle written,
 * strict upper left untouched).  Returns 0, or k+1 if the k-th pivot is not
 * positive. */
int orc_cholesky(int n, double *V) {
  for (int k = 0; k < n; ++k) {
    double d = V[I2(k, k, n)];
    for (int p = 0; p < k; ++p) d -= V[I2(k, p, n)] * V[I2(k, p, n)];
    if (!(d > 0.0)) return k + 1;
    d = sqrt(d);
    V[I2(k, k, n)] = d;
#pragma omp parallel for schedule(static)
    for (int r = k + 1; r < n; ++r) {
      double s = V[I2(r, k, n)];
      for (int p = 0; p < k; ++p) s -= V[I2(r, p, n)] * V[I2(k, p, n)];
      V[I2(r, k, n)] = s / d;
    }
  }
  return 0;
}

/* Forward substitution X = L^{-1} B for B (n x m, column-major, ld n),
 * in place. */
void orc_trsm_lower(int n, int m, const double *L, double *B) {
#pragma omp parallel for schedule(static)
  for (int c = 0; c < m; ++c) {
    double *x = B + I2(0, c, n);
    for (int r = 0; r < n; ++r) {
      double s = x[r];
      for (int p = 0; p < r; ++p) s -= L[I2(r, p, n)] * x[p];
      x[r] = s / L[I2(r, r, n)];
    }
  }
}
