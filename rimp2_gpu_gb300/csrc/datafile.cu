// datafile.cu -- the reference's Calpha{1,2}.data files (host code only).
//
// The reference driver reads one Fortran unformatted sequential file per
// fragment (RIMP2.F90:36-63, CalphaOcc at :190, CalphaVV at :229, and the
// known answers at :257-360); generate.F90 writes it (:75-128, :262, :308,
// :333-339).  Each record is framed by 4-byte length markers (the gfortran
// and ifort default).  Records are read and written in that order:
//
//   0 header: nvirt, nocc, noccEOS, nvirtEOS, NBA, nocctot (4-byte integers)
//   1 Calpha(NBA,nvirt,nocc)   2 EVocc(nocc)   3 EVvirt(nvirt)
//   4 UoccEOST(nocc,noccEOS)   5 UvirtT(nvirt,nvirt)   6 UoccT(nocc,nocc)
//   7 UvirtEOST(nvirt,nvirtEOS)
//   [first order] 8 CalphaOcc(NBA,nocc,nocctot)   9 CalphaVV(NBA,nvirt,nvirt)
//   10 toccEOS(nvirt,noccEOS,nvirt,noccEOS)   11 tvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)
//   12 gvirtEOS(nvirtEOS,nocc,nvirtEOS,nocc)  13 goccEOS(nvirt,noccEOS,nvirt,noccEOS)
//   [first order] 14 djik(nvirt,noccEOS,noccEOS,nocctot)
//                 15 blad(nvirtEOS,nocc,nvirtEOS,nvirt)
//
// Records longer than 2^31-1 bytes would need compiler-specific subrecords
// and are rejected.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace rimp2 {
namespace {

constexpr int NREC = 15;  // array records 1..15

// element count of array record r (1-based) for header h
long long record_elems(int r, const int32_t *h) {
  const long long nv = h[0], no = h[1], ne = h[2], ve = h[3], nb = h[4], nt = h[5];
  switch (r) {
    case 1: return nb * nv * no;
    case 2: return no;
    case 3: return nv;
    case 4: return no * ne;
    case 5: return nv * nv;
    case 6: return no * no;
    case 7: return nv * ve;
    case 8: return nb * no * nt;
    case 9: return nb * nv * nv;
    case 10: return nv * ne * nv * ne;
    case 11: return ve * no * ve * no;
    case 12: return ve * no * ve * no;
    case 13: return nv * ne * nv * ne;
    case 14: return nv * ne * ne * nt;
    case 15: return ve * no * ve * nv;
  }
  return 0;
}

const char *record_name(int r) {
  static const char *n[] = {"header",   "Calpha",   "EVocc",    "EVvirt",   "UoccEOST", "UvirtT",
                            "UoccT",    "UvirtEOST", "CalphaOcc", "CalphaVV", "toccEOS",  "tvirtEOS",
                            "gvirtEOS", "goccEOS",  "djik",     "blad"};
  return r >= 0 && r <= NREC ? n[r] : "?";
}

bool first_order_only(int r) { return r == 8 || r == 9 || r == 14 || r == 15; }

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

int read_marker(FILE *f, int32_t *m) { return fread(m, 4, 1, f) == 1 ? 0 : 1; }

// reads one record of exactly `bytes` bytes into dst (dst null: skip it)
int read_record(FILE *f, int r, void *dst, long long bytes, bool *eof) {
  int32_t m0 = 0, m1 = 0;
  if (read_marker(f, &m0)) {
    if (eof && feof(f)) {
      *eof = true;
      return RIMP2_OK;
    }
    set_error("datafile: cannot read the marker of record %d (%s)", r, record_name(r));
    return RIMP2_ERR_ARG;
  }
  if ((long long)m0 != bytes) {
    set_error("datafile: record %d (%s) holds %d bytes, the header implies %lld", r,
              record_name(r), (int)m0, bytes);
    return RIMP2_ERR_ARG;
  }
  if (dst) {
    if (bytes && fread(dst, 1, (size_t)bytes, f) != (size_t)bytes) {
      set_error("datafile: record %d (%s) is truncated", r, record_name(r));
      return RIMP2_ERR_ARG;
    }
  } else if (fseek(f, (long)bytes, SEEK_CUR) != 0) {
    set_error("datafile: cannot skip record %d (%s)", r, record_name(r));
    return RIMP2_ERR_ARG;
  }
  if (read_marker(f, &m1) || m1 != m0) {
    set_error("datafile: record %d (%s) has a bad trailing marker", r, record_name(r));
    return RIMP2_ERR_ARG;
  }
  return RIMP2_OK;
}

int write_record(FILE *f, int r, const void *src, long long bytes) {
  if (bytes > 2147483647LL) {
    set_error("datafile: record %d (%s) of %lld bytes needs Fortran subrecords (unsupported)", r,
              record_name(r), bytes);
    return RIMP2_ERR_UNSUPPORTED;
  }
  const int32_t m = (int32_t)bytes;
  if (fwrite(&m, 4, 1, f) != 1 || (bytes && fwrite(src, 1, (size_t)bytes, f) != (size_t)bytes) ||
      fwrite(&m, 4, 1, f) != 1) {
    set_error("datafile: write of record %d (%s) failed", r, record_name(r));
    return RIMP2_ERR_ARG;
  }
  return RIMP2_OK;
}

bool header_ok(const int32_t *h) {
  for (int k = 0; k < 6; ++k)
    if (h[k] <= 0) return false;
  return true;
}

}  // namespace
}  // namespace rimp2

using namespace rimp2;

extern "C" int rimp2_datafile_header(const char *path, int *hdr) {
  clear_error();
  RIMP2_REQ(path && hdr, "rimp2_datafile_header: null argument");
  File F;
  F.f = fopen(path, "rb");
  RIMP2_REQ(F.f, "rimp2_datafile_header: cannot open %s", path);
  int32_t h[6];
  RIMP2_TRY(read_record(F.f, 0, h, 24, nullptr));
  RIMP2_REQ(header_ok(h), "rimp2_datafile_header: non-positive dimension in %s", path);
  for (int k = 0; k < 6; ++k) hdr[k] = h[k];
  return RIMP2_OK;
}

extern "C" int rimp2_datafile_read(const char *path, int first_order, double *const *arrays) {
  clear_error();
  RIMP2_REQ(path && arrays, "rimp2_datafile_read: null argument");
  File F;
  F.f = fopen(path, "rb");
  RIMP2_REQ(F.f, "rimp2_datafile_read: cannot open %s", path);
  int32_t h[6];
  RIMP2_TRY(read_record(F.f, 0, h, 24, nullptr));
  RIMP2_REQ(header_ok(h), "rimp2_datafile_read: non-positive dimension in %s", path);
  for (int r = 1; r <= NREC; ++r) {
    if (first_order_only(r) && !first_order) continue;
    bool eof = false;
    // the known-answer records (10 on) may be absent: the file may end there
    RIMP2_TRY(read_record(F.f, r, arrays[r - 1], 8 * record_elems(r, h), r >= 10 ? &eof : nullptr));
    if (eof) {
      for (int q = r; q <= NREC; ++q)
        RIMP2_REQ(!arrays[q - 1] || (first_order_only(q) && !first_order),
                  "rimp2_datafile_read: %s ends before record %d (%s)", path, q, record_name(q));
      break;
    }
  }
  return RIMP2_OK;
}

extern "C" int rimp2_datafile_write(const char *path, const int *hdr, int first_order,
                                    const double *const *arrays) {
  clear_error();
  RIMP2_REQ(path && hdr && arrays, "rimp2_datafile_write: null argument");
  int32_t h[6];
  for (int k = 0; k < 6; ++k) h[k] = hdr[k];
  RIMP2_REQ(header_ok(h), "rimp2_datafile_write: non-positive dimension");
  for (int r = 1; r <= 7; ++r)
    RIMP2_REQ(arrays[r - 1], "rimp2_datafile_write: record %d (%s) is required", r,
              record_name(r));
  if (first_order)
    RIMP2_REQ(arrays[7] && arrays[8], "rimp2_datafile_write: first order needs CalphaOcc, CalphaVV");
  File F;
  F.f = fopen(path, "wb");
  RIMP2_REQ(F.f, "rimp2_datafile_write: cannot create %s", path);
  RIMP2_TRY(write_record(F.f, 0, h, 24));
  for (int r = 1; r <= NREC; ++r) {
    if (first_order_only(r) && !first_order) continue;
    if (r >= 10 && !arrays[r - 1]) break;  // known answers end the file where they stop
    RIMP2_TRY(write_record(F.f, r, arrays[r - 1], 8 * record_elems(r, h)));
  }
  RIMP2_REQ(fflush(F.f) == 0, "rimp2_datafile_write: flush of %s failed", path);
  return RIMP2_OK;
}
