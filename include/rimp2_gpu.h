/*
 * rimp2_gpu.h -- C-ABI of the GB300 (sm_103a) RI-MP2 amplitude / energy library.
 *
 * The entry points keep the argument lists of the CONTAINS subroutines of the
 * reference program RIMP2.F90 (januseriksen/rimp2_gpu), so that the existing
 * Fortran driver can call them through iso_c_binding interfaces without
 * changing its arrays:
 *   - integers arrive by reference (Fortran default), arrays are FP64
 *     column-major with the reference's explicit shapes;
 *   - array arguments are HOST pointers; the library copies in and out on its
 *     own stream.  The *_dev variants take DEVICE pointers instead (the
 *     `host_data use_device` idiom of RIMP2.GPU.F90:117,133,171,185,212,243)
 *     and pass sizes by value;
 *   - every entry returns an int status (RIMP2_OK = 0) and never stops the
 *     process; rimp2_last_error_string() describes the last failure.  (The
 *     reference discards every cuBLAS status, RIMP2.GPU.F90:81,119,135.)
 * There is no CPU fallback: on a machine without a usable sm_103 GPU each
 * compute entry returns RIMP2_ERR_NODEV.  The library works on the device
 * that is current at its first compute call (its stream, error word and
 * memory pool settings belong to that device); one process drives one GPU.
 */
#ifndef RIMP2_GPU_H
#define RIMP2_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RIMP2_OK 0
#define RIMP2_ERR_ARG 1     /* invalid dimension or null pointer */
#define RIMP2_ERR_CUDA 2    /* CUDA runtime / launch error */
#define RIMP2_ERR_NOMEM 3   /* device allocation failed */
#define RIMP2_ERR_NODEV 4   /* no usable GPU */
#define RIMP2_ERR_TIMEOUT 5 /* a device-side bounded wait ran out */
#define RIMP2_ERR_UNSUPPORTED 6

#define RIMP2_PREC_FP64 0  /* plain FP64 (DMMA) fused kernel */
#define RIMP2_PREC_SPLIT 1 /* split-precision tcgen05 alpha contraction */

/* ---- library state ----------------------------------------------------- */
/* Message of the last failing call on this thread ("" after success). */
const char *rimp2_last_error_string(void);
/* Library version string. */
const char *rimp2_version(void);
/* Route all work to a caller stream (cudaStream_t, NULL = library stream). */
int rimp2_set_stream(void *stream);
/* Total and free device memory.  Replaces get_dev_mem (cuda_api.cu:5-8,
 * declared in gpu_interfaces.F90:47-53); pointer arguments instead of C++
 * references so that C and Fortran bind(C) callers can use it. */
int rimp2_get_dev_mem(size_t *total, size_t *free_bytes);
/* Number of kernels this library has launched (all entry points). */
long long rimp2_kernel_launch_count(void);
/* Synchronise `stream` (NULL = library stream) and report any device-side
 * failure of earlier *_dev calls (a bounded wait that expired inside a
 * kernel): RIMP2_ERR_TIMEOUT, else RIMP2_OK.  Host-pointer entry points do
 * this themselves before returning. */
int rimp2_sync_status(void *stream);
/* Failure-detection self-test: a one-thread kernel waits on an mbarrier that
 * nothing completes, with the production kernels' bounded-wait code and a
 * budget of budget_cycles SM clocks (<= 1e9).  Expected result:
 * RIMP2_ERR_TIMEOUT, with the library usable afterwards. */
int rimp2_selftest_bounded_wait(long long budget_cycles, void *stream);
/* Numerics self-test of the split epilogue's reciprocal of an energy
 * denominator (hardware approximation plus one Newton-Raphson step): for the
 * n host values d, r[k] receives that reciprocal and ref[k] CUDA's correctly
 * rounded single-precision 1/d (__frcp_rn), both computed on the GPU. */
int rimp2_selftest_rcp_denom(int n, const float *d, float *r, float *ref);
/* Opt-in CUDA-event timing of the split path's phases; rimp2_last_timing
 * fills ms4 = {slicing, energy kernel, reductions, 0} of the last call. */
int rimp2_set_timing(int on);
int rimp2_last_timing(float *ms4);
/* Energy kernel of the last split-form launch: 0 none yet, 1 one-CTA tile
 * kernel (128x128 MMA), 2 paired-CTA kernel (cta_group::2, 256x128 MMA over
 * two occupied pairs, three products per element pair with a per-column
 * diagonal correction).  One-residual-slice fragments use the kernel the
 * shape-bucket kernel table picks (rimp2_set_split_kernel_rule: the paired
 * kernel for enough occupied orbitals and a long enough auxiliary space);
 * RIMP2_PAIR_KERNEL=0 or =1 in the environment overrides that choice. */
int rimp2_last_split_kernel(void);
/* Measured FP64 tensor-op (DMMA) throughput of this GPU in TFLOP/s, the
 * denominator for the plain kernel's roofline fraction: independent DMMA
 * chains on every SM, timed over one launch of at least a second. */
int rimp2_probe_fp64_peak(double *tflops);

/* ---- drop-in subroutines of RIMP2.F90 -----------------------------------
 * Each replaces the subroutine cited beside it; argument names, order and
 * array shapes are the reference's. */

/* RIMP2_calc_toccA (RIMP2.F90:381-417; GPU form RIMP2.GPU.F90:475-517):
 * tocc(i,jL,a,b) = sum_j [sum_al Calpha(al,a,i) Calpha(al,b,j) /
 *                   (EVocc(i)+EVocc(j)-EVvirt(b)-EVvirt(a))] UoccEOST(j,jL) */
int rimp2_calc_tocca(const int *nvirt, const int *nocc, const int *noccEOS, const int *NBA,
                     const double *Calpha, const double *EVocc, const double *EVvirt,
                     double *tocc, const double *UoccEOST);

/* RIMP2_calc_tvirtA (RIMP2.F90:419-453; GPU RIMP2.GPU.F90:519-559):
 * tvirt(i,j,aL,b) = sum_a [g/D](i,j,a,b) UvirtEOST(a,aL) */
int rimp2_calc_tvirta(const int *nvirt, const int *nocc, const int *nvirtEOS, const int *NBA,
                      const double *Calpha, const double *EVocc, const double *EVvirt,
                      double *tvirt, const double *UvirtEOST);

/* RIMP2_calc_toccB (RIMP2.F90:456-481; GPU RIMP2.GPU.F90:562-592):
 * toccEOS(aL,iL,bL,jL) = sum_A tocc(iL,jL,A,bL) UvirtT(A,aL) */
int rimp2_calc_toccb(const int *nvirt, const int *noccEOS, const double *tocc,
                     const double *UvirtT, double *toccEOS);

/* RIMP2_calc_tvirtB (RIMP2.F90:483-508; GPU RIMP2.GPU.F90:594-623):
 * tvirtEOS(aL,iL,bL,jL) = sum_J tvirt(iL,J,aL,bL) UoccT(J,jL) */
int rimp2_calc_tvirtb(const int *nvirtEOS, const int *nocc, const double *tvirt,
                      const double *UoccT, double *tvirtEOS);

/* RIMP2_TransAlpha1 (RIMP2.F90:510-533; GPU RIMP2.GPU.F90:625-650):
 * AlphaCD5(al,bL,jL) = sum_B UvirtT(B,bL) AlphaCD4(al,B,jL) */
int rimp2_transalpha1(const int *nvirt, const int *noccEOS, const int *nba, const double *UvirtT,
                      const double *AlphaCD4, double *AlphaCD5);

/* RIMP2_TransAlpha2 (RIMP2.F90:536-560; GPU RIMP2.GPU.F90:652-679):
 * AlphaCD5(al,n3,n2) = sum_n1 U(n1,n3) AlphaCD4(al,n1,n2) */
int rimp2_transalpha2(const int *n2, const int *n1, const int *n3, const int *nba,
                      const double *U, const double *AlphaCD4, double *AlphaCD5);

/* RIMP2_calc_gocc (RIMP2.F90:562-587; GPU RIMP2.GPU.F90:707-736):
 * goccEOS(aL,iL,bL,jL) = sum_al Calpha3(al,aL,iL) Calpha3(al,bL,jL) */
int rimp2_calc_gocc(const int *nvirt, const int *noccEOS, const int *NBA, const double *Calpha3,
                    double *goccEOS);

/* RIMP2_calc_gvirt (RIMP2.F90:589-614; GPU RIMP2.GPU.F90:738-766) */
int rimp2_calc_gvirt(const int *nvirtEOS, const int *nocc, const int *NBA, const double *Calpha3,
                     double *gvirtEOS);

/* RIMP2_calc_gen4DimFO (RIMP2.F90:616-641; RIMP2.GPU.F90:768-793):
 * djik(a,b,c,d) = sum_al Calpha3(al,a,b) Calpha4(al,c,d) */
int rimp2_calc_gen4dimfo(const int *NBA, const double *Calpha3, const int *n1, const int *n2,
                         const double *Calpha4, const int *n3, const int *n4, double *djik);

/* Column-major DGEMM as called by the driver at RIMP2.F90:79,87,110,118,137,
 * 160 (cublasDgemm_v2 at RIMP2.GPU.F90:119,135,172,186,213,244, bound in
 * gpu_interfaces.F90:25-33).  transa/transb: 'N' or 'T'.  Hand-written FP64
 * kernel, no cuBLAS. */
int rimp2_dgemm(const char *transa, const char *transb, const int *m, const int *n, const int *k,
                const double *alpha, const double *A, const int *lda, const double *B,
                const int *ldb, const double *beta, double *C, const int *ldc);

/* Driver Steps 5-8 in one call (RIMP2.F90:71-170 with first_order=.false.):
 * toccEOS(nvirt,noccEOS,nvirt,noccEOS), tvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc),
 * goccEOS(nvirt,noccEOS,nvirt,noccEOS), gvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc).
 * All intermediates stay on the device. */
int rimp2_steps5to8(const int *nvirt, const int *nocc, const int *noccEOS, const int *nvirtEOS,
                    const int *NBA, const double *Calpha, const double *EVocc,
                    const double *EVvirt, const double *UoccEOST, const double *UvirtT,
                    const double *UoccT, const double *UvirtEOST, double *toccEOS,
                    double *tvirtEOS, double *goccEOS, double *gvirtEOS);

/* First-order property integrals (RIMP2.F90:172-251, the driver's
 * first_order = .TRUE. block, RIMP2.F90:65):
 *   djik(nvirt,noccEOS,noccEOS,nocctot) from Calpha, UoccEOST, UvirtT and
 *     CalphaOcc(NBA,nocc,nocctot) transformed by UoccallT(nocctot,nocctot);
 *   blad(nvirtEOS,nocc,nvirtEOS,nvirt) from Calpha, UoccT, UvirtEOST and
 *     CalphaVV(NBA,nvirt,nvirt) transformed by UvirtT.
 * The driver passes UoccT(nocc,nocc) as UoccallT (RIMP2.F90:197), which is
 * the same matrix when nocctot = nocc.  As in the driver, the CalphaVV DGEMM
 * sums over the first nocc rows of UvirtT read with leading dimension nocc
 * (RIMP2.F90:232-235: K = ldb = nocc), so the results equal the reference's.
 * All intermediates stay on the device. */
int rimp2_first_order(const int *nvirt, const int *nocc, const int *noccEOS, const int *nvirtEOS,
                      const int *nocctot, const int *NBA, const double *Calpha,
                      const double *CalphaOcc, const double *CalphaVV, const double *UoccEOST,
                      const double *UvirtT, const double *UoccT, const double *UoccallT,
                      const double *UvirtEOST, double *djik, double *blad);

/* DEC fragment energies for general local orbitals, fused (no four-index
 * array is formed).  With the inputs of rimp2_steps5to8 (RIMP2.F90:71-170):
 *   Eocc  = sum toccEOS(aL,iL,bL,jL) (2 goccEOS(aL,iL,bL,jL) - goccEOS(bL,iL,aL,jL))
 *   Evirt = sum tvirtEOS(aL,iL,bL,jL) (2 gvirtEOS(aL,iL,bL,jL) - gvirtEOS(aL,jL,bL,iL))
 * (occupied and virtual partitioning of the fragment energy).  Both equal
 *   sum_ij,ab g_ij^ab / D_ij^ab (2 gt_ij^ab - gt_ij^ba)
 * where gt is the alpha contraction of Calpha projected on both orbital
 * indices: Ct(:,a,i) = sum_ck Pv(a,c) Calpha(:,c,k) Po(k,i) with
 * Po = UoccEOST UoccEOST^T, Pv = UvirtT UvirtT^T (occupied partitioning) or
 * Po = UoccT UoccT^T, Pv = UvirtEOST UvirtEOST^T (virtual partitioning).
 * With U = I both are the canonical MP2 energy.  precision: RIMP2_PREC_FP64
 * (FP64 DMMA) or RIMP2_PREC_SPLIT (tcgen05 split form with the slice count of
 * the shape-bucket table; relative error within 1e-7).  Ct is formed with
 * FP64 GEMMs either way. */
int rimp2_energy_eos(const int *nvirt, const int *nocc, const int *noccEOS, const int *nvirtEOS,
                     const int *NBA, const double *Calpha, const double *EVocc,
                     const double *EVvirt, const double *UoccEOST, const double *UvirtT,
                     const double *UoccT, const double *UvirtEOST, double *Eocc, double *Evirt,
                     const int *precision);

/* ---- Calpha{1,2}.data files (host only) -----------------------------------
 * The reference's fragment files: Fortran unformatted sequential records
 * with 4-byte length markers, read by RIMP2.F90:36-63,190,229,257-360 and
 * written by generate.F90:75-128,262,308,333-339.  Array records in order
 * (arrays[k] is record k+1): Calpha, EVocc, EVvirt, UoccEOST, UvirtT, UoccT,
 * UvirtEOST, CalphaOcc, CalphaVV, toccEOS, tvirtEOS, gvirtEOS, goccEOS,
 * djik, blad; CalphaOcc, CalphaVV, djik and blad exist only in first-order
 * files.  hdr = {nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot}.  Reading: a
 * NULL array skips its record; the known answers (toccEOS on) may be absent
 * if their pointers are NULL.  Writing: the file ends at the first NULL
 * known-answer array.  Records above 2^31-1 bytes: RIMP2_ERR_UNSUPPORTED. */
int rimp2_datafile_header(const char *path, int *hdr);
int rimp2_datafile_read(const char *path, int first_order, double *const *arrays);
int rimp2_datafile_write(const char *path, const int *hdr, int first_order,
                         const double *const *arrays);

/* ---- energies (no counterpart in the reference: the reference stops at the
 * amplitudes toccEOS/tvirtEOS and integrals goccEOS/gvirtEOS; the energy is
 * the closed-shell MP2 expression built from the same g and denominator as
 * RIMP2_calc_toccA, RIMP2.F90:397-404) --------------------------------------
 * e_ij = sum_ab t_ij^ab (2 g_ij^ab - g_ij^ba),  t = g / (e_i+e_j-e_a-e_b),
 * Epair(nocc,nocc) symmetric, Etot = sum_ij e_ij.
 * precision: RIMP2_PREC_FP64 (FP64 DMMA, 1e-11 of the FP64 oracle) or
 * RIMP2_PREC_SPLIT (FP16 Ozaki slices on tcgen05: every pair energy and the
 * total within 1e-7 relative of FP64; the integer part of each product is
 * accumulated exactly, the corrections in FP32, the epilogue in FP32 with
 * double-float denominators and FP64 reductions).  tamp (optional, may be
 * NULL, FP64 path only) receives t(a,i,b,j) in layout (nvirt,nocc,nvirt,nocc). */
int rimp2_energy(const int *nvirt, const int *nocc, const int *NBA, const double *Calpha,
                 const double *EVocc, const double *EVvirt, double *Epair, double *Etot,
                 double *tamp, const int *precision);

/* Same with device pointers and by-value sizes, on `stream` (NULL = library
 * stream).  Stream-ordered; does not synchronise (see rimp2_sync_status). */
int rimp2_energy_dev(int nvirt, int nocc, int NBA, const double *dCalpha, const double *dEVocc,
                     const double *dEVvirt, double *dEpair, double *dEtot, double *dtamp,
                     int precision, void *stream);

/* Residual-slice count the split form uses for a fragment of this shape
 * (the per-shape-bucket choice that holds the energy error within 1e-7). */
int rimp2_split_nslices(int nvirt, int nocc, int NBA);

/* FP64 pair and total energies like rimp2_energy_dev(..., RIMP2_PREC_FP64),
 * for callers that cannot allocate device memory when they call -- a
 * Fortran/OpenACC program whose data regions already hold (nearly) all of the
 * device memory, or code running while another allocator owns it.  It uses
 * no cudaMalloc/cudaFree or allocating library routine, only a fixed 16 MiB
 * device array inside this library (held on every GPU that loads it until the
 * process exits).  Fragments whose pair list plus per-tile partials exceed it
 * (8*npairs*(ceil(nvirt/64)(ceil(nvirt/64)+1)/2 + 1) bytes, npairs =
 * nocc(nocc+1)/2; nocc=128 with nvirt=1024 fits) get RIMP2_ERR_ARG.  stream
 * NULL = the default stream.  Calls share the array: calls that overlap on
 * the GPU race.  The array and this path's kernels are placed on a device by
 * the first call of any entry point of this library there (rimp2_get_dev_mem
 * is a cheap one): make that call before filling the device memory and before
 * any stream capture.  No counterpart in the reference. */
int rimp2_energy_fp64_noalloc_dev(int nvirt, int nocc, int NBA, const double *dCalpha,
                                  const double *dEVocc, const double *dEVvirt, double *dEpair,
                                  double *dEtot, void *stream);

/* Split form with an explicit slice count (1 = S0+R1, 2 = S0+R1+R2; 0 = the
 * plain FP64 kernel, the table's tier for tiny fragments). */
int rimp2_energy_split_dev(int nvirt, int nocc, int NBA, const double *dCalpha,
                           const double *dEVocc, const double *dEVvirt, double *dEpair,
                           double *dEtot, int nslices, void *stream);

/* Many DEC fragments of uneven size in one call.  Fragment f has sizes
 * nocc[f], nvirt[f], NBA[f]; its Calpha/EVocc/EVvirt start at the given
 * element offsets into the concatenated host arrays; Epair of fragment f
 * starts at epair_off[f] (nocc[f]^2 entries), Etot[f] is its total.  The
 * fragments are copied to the device launch group by launch group (the
 * group with the least Calpha first) on the library's copy stream, and each
 * group's kernels wait only for its own fragments: with Calpha in pinned
 * host memory the copies are asynchronous and the transfer of later groups
 * overlaps the kernels of earlier ones (pageable memory is copied through
 * the driver's staging, before the kernels start). */
int rimp2_energy_batched(const int *nfrag, const int *nocc, const int *nvirt, const int *NBA,
                         const double *Calpha, const long long *calpha_off, const double *EVocc,
                         const long long *eo_off, const double *EVvirt, const long long *ev_off,
                         double *Epair, const long long *epair_off, double *Etot,
                         const int *precision);

/* Batched energies of many fragments of uneven size, all resident on the
 * device, in ONE persistent launch per kernel group (one residual slice on
 * the paired-CTA kernel or on the one-CTA kernel, per the kernel table of
 * rimp2_set_split_kernel_rule; two residual slices; plain FP64): a device-side queue of
 * (fragment, pair, tile pair) work items ordered heaviest fragment first,
 * drained by one CTA (pair of CTAs) per SM (pair of SMs).  nslices[f] = 1 or 2 runs
 * fragment f in the split form with that many residual slices; 0 runs it in
 * plain FP64 (the fused DMMA kernel's tile pairs, drained by one persistent
 * launch over all FP64 fragments of the plan).  With use_graph != 0 the
 * whole evaluation (slicing, energy kernels, reductions) is captured once
 * as a CUDA graph and every execute is one graph launch.  nslices may be NULL
 * (per-fragment choice from the shape-bucket table).  The plan keeps its
 * workspace until destroyed and reads the fragment pointers at every
 * execute.  No counterpart in the reference (one fragment per driver run,
 * RIMP2.F90:36-377). */
int rimp2_batch_plan_create(void **plan, int nfrag, const int *nocc, const int *nvirt,
                            const int *NBA, const double *const *dCalpha,
                            const double *const *dEVocc, const double *const *dEVvirt,
                            double *const *dEpair, double *const *dEtot, const int *nslices,
                            int use_graph, void *stream);
int rimp2_batch_plan_execute(void *plan, void *stream);
int rimp2_batch_plan_destroy(void *plan);
/* Shape-bucket table of the split form: fragments with nvirt >= nvirt_min[k]
 * (largest such k) use nslices[k] residual slices (autotuner output); 0 runs
 * the fragment in FP64 (the default table does so below 16 virtuals, where a
 * pair energy has too few (a,b) terms to average the split form's error).
 * Every split-precision entry point follows the table. */
int rimp2_set_split_buckets(int n, const int *nvirt_min, const int *nslices);
/* Energy-kernel table of the one-residual-slice split form: fragments with
 * nvirt >= nvirt_min[k] (largest such k) run the paired-CTA kernel (256-row
 * tiles on a pair of SMs, three FP16 products per element pair) when nocc >=
 * min_nocc[k] and NBA >= min_nba[k], else the one-CTA kernel (128-row tiles,
 * four products).  Default: the autotuner's measured thresholds.  The
 * environment variable RIMP2_PAIR_KERNEL=0 or =1 overrides the table. */
int rimp2_set_split_kernel_rule(int n, const int *nvirt_min, const int *min_nocc,
                                const int *min_nba);
/* Energy kernel a fragment of this shape runs in the split form with the
 * current tables: 0 FP64 tier, 1 one-CTA kernel, 2 paired-CTA kernel. */
int rimp2_split_kernel_for(int nvirt, int nocc, int NBA);

/* ---- synthetic fragments (benchmark / test inputs; no counterpart in the
 * reference, whose fixtures are constants written by generate.F90) --------
 * Seeded Philox4x32-10 + Box-Muller on the device:
 * Calpha(al,a,i) = N(0,1)*0.03/sqrt(1+al/64), EVocc sorted U[-1.5,-0.3],
 * EVvirt sorted U[0.1,3.0].  Any output pointer may be NULL to skip it. */
int rimp2_gen_fragment_dev(unsigned long long seed, int nocc, int nvirt, int NBA, double *dCalpha,
                           double *dEVocc, double *dEVvirt, void *stream);

/* ---- AO front end (no counterpart in the reference, whose input is already
 * Calpha, RIMP2.F90:48-49) --------------------------------------------------
 * Calpha(al,a,i) = sum_be Linv(al,be) sum_{mu,nu} Cmo(mu,nocc+a) Cmo(nu,i) ao(be,mu,nu)
 * with V = L L^T the Cholesky factorisation of the auxiliary metric.  All
 * FP64 on the GPU.  ao(NBA,nbas,nbas) symmetric in (mu,nu), V(NBA,NBA) SPD,
 * Cmo(nbas,nbas) columns occ then virt; Calpha out (NBA,nvirt,nocc). */
int rimp2_calpha_from_ao(const int *NBA, const int *nbas, const int *nocc, const int *nvirt,
                         const double *ao, const double *V, const double *Cmo, double *Calpha);
/* Device-pointer form on `stream` (synchronises once: the metric's
 * positive-definiteness is checked before the solve). */
int rimp2_calpha_from_ao_dev(int NBA, int nbas, int nocc, int nvirt, const double *dao,
                             const double *dV, const double *dCmo, double *dCalpha, void *stream);
/* Same, with the AO->MO transform on the tcgen05 tensor cores (exact-integer
 * FP16 slices with two residual slices; Calpha within ~1e-8 of the FP64
 * form); the metric Cholesky and the triangular solve stay FP64.  For
 * nocc <= 80 its first half contracts over the middle AO index, relying on
 * the (mu,nu) symmetry of ao stated above. */
int rimp2_calpha_from_ao_split_dev(int NBA, int nbas, int nocc, int nvirt, const double *dao,
                                   const double *dV, const double *dCmo, double *dCalpha,
                                   void *stream);
/* Building blocks: the AO->MO transform alone, (alpha|a i) in the Calpha
 * layout (NBA,nvirt,nocc); split != 0 selects the tensor-core form (which,
 * for nocc <= 80, uses the (mu,nu) symmetry of ao). */
int rimp2_ao2mo_dev(int NBA, int nbas, int nocc, int nvirt, const double *dao, const double *dCmo,
                    double *dout, int split, void *stream);
/* Lower Cholesky V = L L^T in place (n x n, strict upper
 * zeroed; RIMP2_ERR_ARG if not positive definite) and X = L^{-1} B
 * (B n x m, overwritten as workspace; X separate). FP64, blocked, GPU. */
int rimp2_cholesky_dev(int n, double *dV, void *stream);
int rimp2_trsm_lower_dev(int n, int m, const double *dL, double *dB, double *dX, void *stream);
/* Synthetic AO inputs on the device: (alpha|mu nu) = N(0,1) exp(-|mu-nu|/32),
 * symmetric in (mu,nu); V = A A^T/NBA + 0.1 I with A ~ N(0,1).  Either
 * output may be NULL. */
int rimp2_gen_ao_dev(unsigned long long seed, int NBA, int nbas, double *dao, double *dV,
                     void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RIMP2_GPU_H */
