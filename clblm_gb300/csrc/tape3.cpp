// tape3.cpp -- reader of LNFL's binary line file (TAPE3), the file CLBLM's
// RDLIN reads (clblm_ODLAY.f90:2571-2798) through CLBLM_LineData
// (clblm_LineData.f90:52-161).  Host code only.
//
// The file is Fortran unformatted sequential: every record is framed by its
// byte length as a 4-byte integer before and after it.  Records:
//   1. the file header (HLINID(10) char*8, BMOLID(64) char*8, MOLCNT, MCNTLC,
//      MCNTNL (64 int32 each), SUMSTR(64) real32, LINMOL, FLINLO, FLINHI,
//      LINCNT, ILINLC, ILINNL, IREC, IRECTL, HID1(2) char*8)
//   2. if the 8th character of HLINID(7) is '^': N_NEGEPP(64), N_RESETEPP(64),
//      XSPACE(4096) -- skipped
//   then per block of up to 250 lines: the panel header INPUT_HEADER
//   (VMIN, VMAX real64, NREC, NWDS int32) and INPUT_BLOCK (VNU(250) real64;
//   SP, ALFA, EPP real32; MOL int32; HWHM, TMPALF, PSHIFT real32; IFLG
//   int32; broadening and speed-dependence data, not used on this path).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/clblm_gb300.h"

namespace {

constexpr int kRec = CLBLM_LINES_PER_RECORD;

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

// one Fortran record into buf; returns false at the end of the file
bool read_record(FILE* f, std::vector<unsigned char>* buf, std::string* err) {
  int32_t n1 = 0, n2 = 0;
  size_t got = fread(&n1, 4, 1, f);
  if (got != 1) return false;
  if (n1 < 0 || n1 > (1 << 28)) {
    *err = "bad record length";
    return false;
  }
  buf->resize((size_t)n1);
  if (n1 > 0 && fread(buf->data(), 1, (size_t)n1, f) != (size_t)n1) {
    *err = "truncated record";
    return false;
  }
  if (fread(&n2, 4, 1, f) != 1 || n2 != n1) {
    *err = "record markers do not match";
    return false;
  }
  return true;
}

template <typename T>
T at(const std::vector<unsigned char>& b, size_t off) {
  T v;
  std::memcpy(&v, b.data() + off, sizeof v);
  return v;
}

}  // namespace

extern "C" int clblm_tape3_read(const char* path, double v1, double v2, clblm_lines_t* lines, int64_t cap,
                                int64_t* n_lines, char* errbuf, int32_t errlen) {
  auto fail = [&](int code, const std::string& msg) {
    if (errbuf && errlen > 0) {
      std::snprintf(errbuf, (size_t)errlen, "%s", msg.c_str());
    }
    return code;
  };
  if (!path || !n_lines) return fail(CLBLM_ERR_ARG, "null argument");
  File F;
  F.f = std::fopen(path, "rb");
  if (!F.f) return fail(CLBLM_ERR_ARG, std::string("cannot open ") + path);
  std::vector<unsigned char> b;
  std::string err;
  if (!read_record(F.f, &b, &err)) return fail(CLBLM_ERR_ARG, "no file header: " + err);
  const size_t kHeader = 80 + 512 + 4 * 64 * 4 + 4 * 8 + 16;
  if (b.size() < kHeader) return fail(CLBLM_ERR_ARG, "file header too short");
  if (b[6 * 8 + 7] == '^') {  // HLINID(7)(8:8): the negative-EPP record follows
    if (!read_record(F.f, &b, &err)) return fail(CLBLM_ERR_ARG, "missing negative-EPP record: " + err);
  }
  const bool fill = lines && lines->vnu;
  int64_t n = 0;
  bool partial = false;  // a block of fewer than 250 lines was kept
  for (;;) {
    if (!read_record(F.f, &b, &err)) {
      if (!err.empty()) return fail(CLBLM_ERR_ARG, "panel header: " + err);
      break;
    }
    if (b.size() < 24) return fail(CLBLM_ERR_ARG, "panel header too short");
    const double vmin = at<double>(b, 0), vmax = at<double>(b, 8);
    const int32_t nrec = at<int32_t>(b, 16);
    if (nrec < 0 || nrec > kRec) return fail(CLBLM_ERR_ARG, "NREC beyond 250 (RDLIN: NREC GT LIMIN)");
    if (!read_record(F.f, &b, &err)) return fail(CLBLM_ERR_ARG, "line block: " + err);
    if (b.size() < (size_t)kRec * (8 + 8 * 4)) return fail(CLBLM_ERR_ARG, "line block too short");
    if (vmax < v1 || vmin > v2) continue;  // whole records outside the window
    if (partial)
      return fail(CLBLM_ERR_UNSUPPORTED,
                  "a block of fewer than 250 lines is followed by more lines: the line list keeps records of 250");
    if (nrec < kRec) partial = true;
    if (fill) {
      if (n + nrec > cap) return fail(CLBLM_ERR_CAPACITY, "more lines than the capacity");
      const size_t o_sp = 8 * kRec, o_alfa = o_sp + 4 * kRec, o_epp = o_alfa + 4 * kRec, o_mol = o_epp + 4 * kRec;
      const size_t o_hwhm = o_mol + 4 * kRec, o_tmp = o_hwhm + 4 * kRec, o_psh = o_tmp + 4 * kRec;
      const size_t o_iflg = o_psh + 4 * kRec;
      for (int i = 0; i < nrec; ++i) {
        const int64_t k = n + i;
        const_cast<double*>(lines->vnu)[k] = at<double>(b, 8 * (size_t)i);
        const_cast<float*>(lines->sp)[k] = at<float>(b, o_sp + 4 * (size_t)i);
        const_cast<float*>(lines->alfa)[k] = at<float>(b, o_alfa + 4 * (size_t)i);
        const_cast<float*>(lines->epp)[k] = at<float>(b, o_epp + 4 * (size_t)i);
        const_cast<int32_t*>(lines->mol)[k] = at<int32_t>(b, o_mol + 4 * (size_t)i);
        const_cast<float*>(lines->hwhm)[k] = at<float>(b, o_hwhm + 4 * (size_t)i);
        const_cast<float*>(lines->tmpalf)[k] = at<float>(b, o_tmp + 4 * (size_t)i);
        const_cast<float*>(lines->pshift)[k] = at<float>(b, o_psh + 4 * (size_t)i);
        const_cast<int32_t*>(lines->iflg)[k] = at<int32_t>(b, o_iflg + 4 * (size_t)i);
      }
    }
    n += nrec;
  }
  *n_lines = n;
  if (fill) lines->n = n;
  return CLBLM_OK;
}
