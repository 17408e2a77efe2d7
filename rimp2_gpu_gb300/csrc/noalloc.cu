// noalloc.cu -- FP64 pair/total energy entry point that allocates nothing.
//
// Why: some callers cannot allocate device memory at the point where they
// need an energy -- a Fortran/OpenACC host program that has already handed
// (nearly) all device memory to its own data regions, code that runs while
// another library owns the CUDA memory pool, or a caller that must not
// trigger allocator work mid-computation.  For them the library keeps its
// working memory for this one path in a fixed, file-scope device array that
// exists from the moment the library's module is loaded until the process
// exits (on every GPU that loads it).
//
// Limit: NOALLOC_SCRATCH_BYTES = 16 MiB, holding the (i<=j) pair list and one
// FP64 partial energy per (pair, 64x64 tile pair) work item:
//   8*npairs*ntp + 8*npairs (+alignment) <= 16 MiB,
//   npairs = nocc(nocc+1)/2, ntp = t(t+1)/2, t = ceil(nvirt/64).
// nocc=128, nvirt=1024 needs 9.1 MB; larger fragments are rejected with
// RIMP2_ERR_ARG and a message.
//
// Contract: every call shares the one array and it keeps the last call's
// contents; each launch writes every scratch element it later reads (pair
// list, partials), so nothing needs clearing between calls.  Calls whose
// work overlaps on the GPU (different streams, or different host threads on
// one device) race on the array: serialise them.
//
// When the array exists: CUDA loads a module (and creates its __device__
// arrays) lazily, when something first refers to it.  The library's regular
// device set-up (ensure_device, run by the first call of any other entry
// point, rimp2_get_dev_mem included) loads this array and the four kernels
// of this path on the current device.  A caller that must not allocate later
// makes such a call once per device before it fills the device memory (and
// before any stream capture); if the allocation-free entry point is the first
// call on a device, that call loads them itself.
#include "common.cuh"

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array on the current device.  The name
// g_noalloc_scratch is only a host-side handle; kernels must be given this
// address, never the symbol itself.  Looked up on every call (cheap once the
// module is loaded), so a device reset that reloads the module at another
// address leaves no stale pointer behind.
int scratch_address(void **out) {
  int dev = 0;
  RIMP2_CK(cudaGetDevice(&dev));
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    (void)cudaGetLastError();
    rimp2::set_error("cudaGetSymbolAddress(scratch) failed on device %d: %s", dev,
                     cudaGetErrorString(e));
    return RIMP2_ERR_CUDA;
  }
  *out = p;
  return RIMP2_OK;
}

// Device check without the library's lazily allocated state.
int check_device_noalloc() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    (void)cudaGetLastError();
    rimp2::set_error("no CUDA device available; this library has no CPU path");
    return RIMP2_ERR_NODEV;
  }
  int dev = 0, major = 0, minor = 0;
  RIMP2_CK(cudaGetDevice(&dev));
  RIMP2_CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  RIMP2_CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
  if (!(major == 10 && minor == 3)) {
    rimp2::set_error("device is sm_%d%d; this library is built for sm_103a only", major, minor);
    return RIMP2_ERR_NODEV;
  }
  return RIMP2_OK;
}

}  // namespace

namespace rimp2 {
int noalloc_preload() {
  void *p = nullptr;
  RIMP2_TRY(scratch_address(&p));
  return preload_plain_scratch_kernels();
}
}  // namespace rimp2

extern "C" int rimp2_energy_fp64_noalloc_dev(int nvirt, int nocc, int NBA, const double *dCalpha,
                                             const double *dEVocc, const double *dEVvirt,
                                             double *dEpair, double *dEtot, void *stream) {
  rimp2::clear_error();
  RIMP2_REQ(nvirt > 0 && nocc > 0 && NBA > 0, "rimp2_energy_fp64_noalloc_dev: bad dims");
  RIMP2_REQ(dCalpha && dEVocc && dEVvirt && dEpair && dEtot,
            "rimp2_energy_fp64_noalloc_dev: null array");
  long long npairs = 0, nitems = 0;
  rimp2::plain_energy_scratch_sizes(nvirt, nocc, &npairs, &nitems);
  const size_t pairs_bytes = ((size_t)(2 * npairs) * sizeof(int) + 255) & ~(size_t)255;
  const size_t need = pairs_bytes + (size_t)nitems * sizeof(double);
  RIMP2_REQ(nitems <= 2147483647LL && need <= NOALLOC_SCRATCH_BYTES,
            "rimp2_energy_fp64_noalloc_dev: fragment nocc=%d nvirt=%d needs %zu bytes of scratch, "
            "above the fixed %zu-byte limit of this allocation-free entry point",
            nocc, nvirt, need, NOALLOC_SCRATCH_BYTES);
  RIMP2_TRY(check_device_noalloc());
  void *base = nullptr;
  RIMP2_TRY(scratch_address(&base));
  RIMP2_TRY(rimp2::preload_plain_scratch_kernels());
  rimp2::PlainEnergyArgs a;
  a.Ca = dCalpha;
  a.NBA = NBA;
  a.nvirt = nvirt;
  a.nocc = nocc;
  a.eo = dEVocc;
  a.ev = dEVvirt;
  a.Epair = dEpair;
  a.Etot = dEtot;
  a.tamp = nullptr;
  a.pairs = nullptr;
  a.npairs = 0;
  int *pairs = static_cast<int *>(base);
  double *part = reinterpret_cast<double *>(static_cast<unsigned char *>(base) + pairs_bytes);
  return rimp2::plain_energy_f64_scratch(a, pairs, part, (cudaStream_t)stream);
}
