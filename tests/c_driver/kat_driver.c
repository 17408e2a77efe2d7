/* C driver of the C-ABI (include/rimp2_gpu.h), written the way a host
 * program in C would call the library: the reference's constant fixtures of
 * generate.F90:77-128 (first shipped size: nvirt 74, nocc 10, noccEOS 4,
 * nvirtEOS 15, NBA 273) through rimp2_steps5to8, checked against their closed
 * forms with the reference's own 1e-10 test (RIMP2.F90:262), and the MP2
 * energy of the same Calpha in FP64 and split precision.
 *
 * Exit status: 0 all checks passed, 2 no usable GPU (RIMP2_ERR_NODEV, the
 * expected result on a machine without one), 1 any failure. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "rimp2_gpu.h"

static double *alloc(size_t n) { return (double *)calloc(n, sizeof(double)); }

int main(void) {
  int nvirt = 74, nocc = 10, noccEOS = 4, nvirtEOS = 15, NBA = 273;
  size_t nv = nvirt, no = nocc, ne = noccEOS, ve = nvirtEOS, nb = NBA;
  double *Ca = alloc(nb * nv * no), *eo = alloc(no), *ev = alloc(nv);
  double *UoE = alloc(no * ne), *UvT = alloc(nv * nv), *UoT = alloc(no * no), *UvE = alloc(nv * ve);
  /* generate.F90:81-125 (1-based formulas, A*x/A kept as written there) */
  for (int c = 1; c <= nocc; ++c)
    for (int b = 1; b <= nvirt; ++b)
      for (int a = 1; a <= NBA; ++a)
        Ca[(a - 1) + nb * ((b - 1) + nv * (c - 1))] =
            a * 0.00124235636 / a + b * 0.01010101 / b + c * 0.014321 / c;
  for (int c = 1; c <= nocc; ++c) eo[c - 1] = c * 1.934321 / c;
  for (int c = 1; c <= nvirt; ++c) ev[c - 1] = c * 1.91321 / c;
  for (int b = 1; b <= noccEOS; ++b)
    for (int a = 1; a <= nocc; ++a) UoE[(a - 1) + no * (b - 1)] = a * 0.030321 / a + b * 0.101121 / b;
  for (int b = 1; b <= nvirt; ++b)
    for (int a = 1; a <= nvirt; ++a) UvT[(a - 1) + nv * (b - 1)] = a * 0.021321 / a + b * 0.01321 / b;
  for (int b = 1; b <= nocc; ++b)
    for (int a = 1; a <= nocc; ++a) UoT[(a - 1) + no * (b - 1)] = a * 0.032321 / a + b * 0.01521 / b;
  for (int b = 1; b <= nvirtEOS; ++b)
    for (int a = 1; a <= nvirt; ++a) UvE[(a - 1) + nv * (b - 1)] = a * 0.023321 / a + b * 0.01421 / b;

  double *tE = alloc(nv * ne * nv * ne), *vE = alloc(ve * no * ve * no);
  double *gE = alloc(nv * ne * nv * ne), *gvE = alloc(ve * no * ve * no);
  int st = rimp2_steps5to8(&nvirt, &nocc, &noccEOS, &nvirtEOS, &NBA, Ca, eo, ev, UoE, UvT, UoT, UvE,
                           tE, vE, gE, gvE);
  if (st == RIMP2_ERR_NODEV) {
    printf("no usable GPU: %s\n", rimp2_last_error_string());
    return 2;
  }
  if (st != RIMP2_OK) {
    fprintf(stderr, "rimp2_steps5to8: %s\n", rimp2_last_error_string());
    return 1;
  }
  /* closed forms: every element of each array is the same constant */
  const double c0 = 0.00124235636 + 0.01010101 + 0.014321, D = 2 * (1.934321 - 1.91321);
  const double U1 = 0.030321 + 0.101121, UV = 0.021321 + 0.01321;
  const double UO = 0.032321 + 0.01521, W = 0.023321 + 0.01421;
  const double exp_t = NBA * c0 * c0 / D * pow(nocc * U1, 2) * pow(nvirt * UV, 2);
  const double exp_v = NBA * c0 * c0 / D * pow(nvirt * W, 2) * pow(nocc * UO, 2);
  const double exp_g = NBA * pow(c0 * nocc * U1 * nvirt * UV, 2);
  const double exp_gv = NBA * pow(c0 * nocc * UO * nvirt * W, 2);
  double worst = 0.0;
  for (size_t k = 0; k < nv * ne * nv * ne; ++k) {
    worst = fmax(worst, fabs(tE[k] - exp_t));
    worst = fmax(worst, fabs(gE[k] - exp_g));
  }
  for (size_t k = 0; k < ve * no * ve * no; ++k) {
    worst = fmax(worst, fabs(vE[k] - exp_v));
    worst = fmax(worst, fabs(gvE[k] - exp_gv));
  }
  printf("steps 5-8: max |diff| to the closed forms %.3e\n", worst);
  if (!(worst <= 1e-10)) return 1;

  /* MP2 energy of the same Calpha, FP64 and split precision */
  double *Ep = alloc(no * no), *Ep2 = alloc(no * no), E = 0.0, E2 = 0.0;
  int p64 = RIMP2_PREC_FP64, psp = RIMP2_PREC_SPLIT;
  if (rimp2_energy(&nvirt, &nocc, &NBA, Ca, eo, ev, Ep, &E, NULL, &p64) != RIMP2_OK ||
      rimp2_energy(&nvirt, &nocc, &NBA, Ca, eo, ev, Ep2, &E2, NULL, &psp) != RIMP2_OK) {
    fprintf(stderr, "rimp2_energy: %s\n", rimp2_last_error_string());
    return 1;
  }
  /* constant Calpha: every g equals NBA c0^2, every denominator D, so
   * E = nocc^2 nvirt^2 NBA^2 c0^4 / D (each term g (2g - g) / D) */
  const double expE = pow((double)nocc * nvirt * NBA * c0 * c0, 2) / D;
  printf("energy: FP64 %.15e  split %.15e  closed form %.15e\n", E, E2, expE);
  if (!(fabs(E - expE) <= 1e-11 * fabs(expE))) return 1;
  if (!(fabs(E2 - expE) <= 1e-7 * fabs(expE))) return 1;
  printf("ok\n");
  return 0;
}
