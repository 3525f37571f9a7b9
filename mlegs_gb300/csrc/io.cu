// io.cu — field I/O in the reference's file formats (msave / mload, mlegs_scalar_io.f90:6-249) and the
// parameter-file reader (read_input, mlegs_misc_io.f90:307-388).  Host code: the field is copied
// between the device and a host buffer and written or parsed here.
#include "common.cuh"
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace mlg {

// ------------------------------------------------------------------------------------------------
// formatted numbers

// Fortran '1PE24.15E3': one digit before the point, 15 after, a 3-digit exponent, right-justified in
// 24 columns (mlegs_envir.f90:21 sets the width, the fraction digits are the width less 9)
static void right24(const std::string& t, char* out24) {   // right-justified in 24 columns
  size_t L = std::min<size_t>(t.size(), 24);
  std::memset(out24, ' ', 24 - L);
  std::memcpy(out24 + 24 - L, t.data(), L);
  out24[24] = 0;
}
static void fmt_pe(double v, char* out24) {
  if (std::isnan(v)) { right24("NaN", out24); return; }
  if (std::isinf(v)) { right24(v < 0 ? "-Infinity" : "Infinity", out24); return; }
  char m[64];
  std::snprintf(m, sizeof m, "%.15E", v);   // d.dddddddddddddddE+xx (two or more exponent digits)
  char* e = std::strchr(m, 'E');
  int ex = std::atoi(e + 1);
  *e = 0;
  std::string t(m);
  char x[16];
  std::snprintf(x, sizeof x, "%03d", ex < 0 ? -ex : ex);
  t += ex < 0 ? "E-" : "E+";
  t += x;
  right24(t, out24);
}

// a Fortran real literal: D or d exponents are read as E
static bool parse_real(const std::string& t, double* v) {
  std::string u = t;
  for (char& c : u)
    if (c == 'D' || c == 'd') c = 'E';
  char* end = nullptr;
  errno = 0;
  *v = std::strtod(u.c_str(), &end);
  return end && *end == 0 && end != u.c_str() && errno != ERANGE;
}
static bool parse_int(const std::string& t, int* v) {
  char* end = nullptr;
  long x = std::strtol(t.c_str(), &end, 10);
  if (!end || *end != 0 || end == t.c_str()) return false;
  *v = (int)x;
  return true;
}
// a Fortran logical: T, F, .TRUE., .false., t..., f...
static bool parse_logical(const std::string& t, int* v) {
  size_t i = (!t.empty() && t[0] == '.') ? 1 : 0;
  if (i >= t.size()) return false;
  char c = (char)std::toupper((unsigned char)t[i]);
  if (c == 'T') { *v = 1; return true; }
  if (c == 'F') { *v = 0; return true; }
  return false;
}

// ------------------------------------------------------------------------------------------------
// list-directed input: each read starts at a new record, values may continue over records, blank
// records hold no values, and the rest of the last record read is discarded; a slash ends a read
class ListReader {
 public:
  explicit ListReader(FILE* f) : f_(f) {}
  // the next record as it stands (a formatted '(a...)' read)
  bool raw_line(std::string* out) { return next_record(out); }
  // n values (as text) by list-directed rules
  bool read(std::vector<std::string>* vals, size_t n) {
    vals->clear();
    std::string rec;
    while (vals->size() < n) {
      if (!next_record(&rec)) return false;
      size_t i = 0;
      while (i < rec.size() && vals->size() < n) {
        while (i < rec.size() && (rec[i] == ' ' || rec[i] == '\t' || rec[i] == ',' || rec[i] == '\r')) ++i;
        if (i >= rec.size()) break;
        if (rec[i] == '/') {   // a slash ends the read; the items left keep their values (empty here)
          vals->resize(n);
          return true;
        }
        size_t j = i;
        if (rec[i] == '\'' || rec[i] == '"') {
          char q = rec[i];
          j = rec.find(q, i + 1);
          if (j == std::string::npos) j = rec.size();
          vals->push_back(rec.substr(i + 1, j - i - 1));
          i = j + 1;
          continue;
        }
        while (j < rec.size() && rec[j] != ' ' && rec[j] != '\t' && rec[j] != ',' && rec[j] != '/' && rec[j] != '\r') ++j;
        vals->push_back(rec.substr(i, j - i));
        i = j;
      }
    }
    return true;
  }
  bool read1(std::string* v) {
    std::vector<std::string> t;
    if (!read(&t, 1)) return false;
    *v = t[0];
    return true;
  }

 private:
  bool next_record(std::string* out) {
    out->clear();
    int c;
    bool any = false;
    while ((c = std::fgetc(f_)) != EOF) {
      any = true;
      if (c == '\n') return true;
      out->push_back((char)c);
    }
    return any;
  }
  FILE* f_;
};

// ------------------------------------------------------------------------------------------------
// msave / mload

struct FieldFile {
  std::vector<double> e;   // 2 * nrdim * npdim * nzdim, (re, im) interleaved, Fortran order
  double ln = 0.0;
  int off[3] = {0, 0, 0};
  char space[4] = {'P', 'P', 'P', 0};
};

static std::string file_name(const char* fn, int is_global) {
  return is_global ? std::string(fn) : std::string(fn) + "_0";   // the per-rank form of rank 0
}

static int write_binary(FILE* f, const FieldFile& d, const int dims[3], int is_global) {
  int hdr[9] = {dims[0], dims[1], dims[2], dims[0], dims[1], dims[2], 0, 0, 0};
  size_t nh = is_global ? 3 : 9;   // global: sizes; per rank: glb_sz, loc_sz, loc_st
  if (std::fwrite(hdr, sizeof(int), nh, f) != nh) return -1;
  if (std::fwrite(d.e.data(), sizeof(double), d.e.size(), f) != d.e.size()) return -1;
  if (std::fwrite(&d.ln, sizeof(double), 1, f) != 1) return -1;
  if (std::fwrite(d.off, sizeof(int), 3, f) != 3) return -1;
  if (std::fwrite(d.space, 1, 3, f) != 3) return -1;
  return 0;
}

static int write_text(FILE* f, const FieldFile& d, const int dims[3], int is_global) {
  if (is_global) {
    std::fprintf(f, " %10d %10d %10d\n", dims[0], dims[1], dims[2]);
  } else {
    for (int r = 0; r < 3; ++r)
      if (r < 2) std::fprintf(f, " %10d %10d %10d\n", dims[0], dims[1], dims[2]);
      else std::fprintf(f, " %10d %10d %10d\n", 0, 0, 0);
  }
  char buf[32];
  const size_t n1 = dims[0], n2 = dims[1], n3 = dims[2];
  for (size_t k = 0; k < n3; ++k) {
    for (size_t i = 0; i < n1; ++i) {
      for (size_t j = 0; j < n2; ++j) {
        size_t o = 2 * (i + n1 * (j + n2 * k));
        fmt_pe(d.e[o], buf); std::fputs(buf, f);
        fmt_pe(d.e[o + 1], buf); std::fputs(buf, f);
      }
      if (i + 1 < n1) std::fputc('\n', f);
    }
    if (k + 1 < n3) std::fputs("\n\n", f);   // the row's end, then one blank line between z blocks
  }
  std::fputc('\n', f);
  std::fprintf(f, " %.17G %d %d %d\n", d.ln, d.off[0], d.off[1], d.off[2]);
  std::fprintf(f, " %.3s\n", d.space);
  return std::ferror(f) ? -1 : 0;
}

static int read_binary(FILE* f, FieldFile* d, const int dims[3], int is_global) {
  int hdr[9];
  size_t nh = is_global ? 3 : 9;
  if (std::fread(hdr, sizeof(int), nh, f) != nh) return set_error(MLG_EPARAM, "mload_scalar: truncated file");
  const int* sz = is_global ? hdr : hdr + 3;   // the reference checks the local size of a per-rank file
  if (sz[0] != dims[0] || sz[1] != dims[1] || sz[2] != dims[2])
    return set_error(MLG_ESIZE, "mloadc: size inconsistency between data and array");
  d->e.resize(2ull * dims[0] * dims[1] * dims[2]);
  if (std::fread(d->e.data(), sizeof(double), d->e.size(), f) != d->e.size() ||
      std::fread(&d->ln, sizeof(double), 1, f) != 1 || std::fread(d->off, sizeof(int), 3, f) != 3 ||
      std::fread(d->space, 1, 3, f) != 3)
    return set_error(MLG_EPARAM, "mload_scalar: truncated file");
  d->space[3] = 0;
  return 0;
}

// the formatted layout read by values (blank lines and the width of each field do not matter), so
// that files written by either side read back
static int read_text(FILE* f, FieldFile* d, const int dims[3], int is_global) {
  ListReader rd(f);
  std::vector<std::string> t;
  int sz[3];
  for (int r = 0; r < (is_global ? 1 : 3); ++r) {
    if (!rd.read(&t, 3)) return set_error(MLG_EPARAM, "mload_scalar: truncated file");
    if (r == (is_global ? 0 : 1))
      for (int a = 0; a < 3; ++a)
        if (!parse_int(t[a], &sz[a])) return set_error(MLG_EPARAM, "mload_scalar: unreadable size");
  }
  if (sz[0] != dims[0] || sz[1] != dims[1] || sz[2] != dims[2])
    return set_error(MLG_ESIZE, "mloadc: size inconsistency between data and array");
  const size_t n = 2ull * dims[0] * dims[1] * dims[2];
  d->e.assign(n, 0.0);
  const size_t n1 = dims[0], n2 = dims[1];
  size_t got = 0;
  std::vector<double> row;
  while (got < n) {   // one record per (r, z): 2*npdim values
    if (!rd.read(&t, 2 * n2)) return set_error(MLG_EPARAM, "mload_scalar: truncated data");
    size_t rowi = got / (2 * n2);   // = i + n1*k
    size_t i = rowi % n1, k = rowi / n1;
    for (size_t j = 0; j < n2; ++j) {
      double re, im;
      if (!parse_real(t[2 * j], &re) || !parse_real(t[2 * j + 1], &im))
        return set_error(MLG_EPARAM, "mload_scalar: unreadable value");
      size_t o = 2 * (i + n1 * (j + n2 * k));
      d->e[o] = re;
      d->e[o + 1] = im;
    }
    got += 2 * n2;
  }
  if (!rd.read(&t, 4)) return set_error(MLG_EPARAM, "mload_scalar: missing ln and offsets");
  if (!parse_real(t[0], &d->ln) || !parse_int(t[1], &d->off[0]) || !parse_int(t[2], &d->off[1]) ||
      !parse_int(t[3], &d->off[2]))
    return set_error(MLG_EPARAM, "mload_scalar: unreadable ln or offsets");
  std::string sp;
  if (!rd.read1(&sp) || sp.size() < 3) return set_error(MLG_EPARAM, "mload_scalar: missing space tag");
  std::memcpy(d->space, sp.data(), 3);
  d->space[3] = 0;
  return 0;
}

}  // namespace mlg

using namespace mlg;

extern "C" {

int mlg_msave(mlg_scalar h, const char* fn, int is_binary, int is_global) {
  if (!h || !fn) return set_error(MLG_EHANDLE, "msave: null argument");
  int dims[9];
  MLG_TRY(mlg_kit_dims(dims));
  Scalar* s = reinterpret_cast<Scalar*>(h);
  FieldFile d;
  d.e.resize(2ull * dims[0] * dims[1] * dims[2]);
  MLG_TRY(mlg_scalar_download(h, d.e.data(), &d.ln, d.space));
  for (int a = 0; a < 3; ++a) d.off[a] = s->off[a];
  std::string name = file_name(fn, is_global);
  FILE* f = std::fopen(name.c_str(), is_binary ? "wb" : "w");
  if (!f) return set_error(MLG_EPARAM, "msave_scalar: cannot open " + name);
  int rc = is_binary ? write_binary(f, d, dims, is_global) : write_text(f, d, dims, is_global);
  if (std::fclose(f) != 0) rc = -1;
  if (rc) return set_error(MLG_EPARAM, "msave_scalar: write failed on " + name);
  return 0;
}

int mlg_mload(mlg_scalar h, const char* fn, int is_binary, int is_global) {
  if (!h || !fn) return set_error(MLG_EHANDLE, "mload: null argument");
  int dims[9];
  MLG_TRY(mlg_kit_dims(dims));
  std::string name = file_name(fn, is_global);
  FILE* f = std::fopen(name.c_str(), is_binary ? "rb" : "r");
  if (!f) return set_error(MLG_EPARAM, "mload_scalar: cannot open " + name);
  FieldFile d;
  int rc = is_binary ? read_binary(f, &d, dims, is_global) : read_text(f, &d, dims, is_global);
  std::fclose(f);
  MLG_TRY(rc);
  MLG_TRY(mlg_scalar_upload(h, d.e.data(), d.ln, d.space));   // the space tag is checked here
  MLG_TRY(mlg_scalar_chop_offset(h, d.off[0], d.off[1], d.off[2]));
  return mlg_sync();
}

// ------------------------------------------------------------------------------------------------
// read_input (mlegs_misc_io.f90:307-388)

static bool dir_ok(const std::string& d) {
  static const char* ok = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ0123456789_./-";
  for (char c : d)
    if (!std::strchr(ok, c)) return false;
  return true;
}
static int mkdir_p(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i < d.size(); ++i) {
    cur.push_back(d[i]);
    if (d[i] == '/' || i + 1 == d.size()) {
      if (cur == "/" || cur == "./" || cur == "../") continue;
      if (::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) return -1;
    }
  }
  return 0;
}
static std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

int mlg_read_input(const char* fn, mlg_params* p, mlg_run_params* run, int make_dirs) {
  if (!fn || !p || !run) return set_error(MLG_EHANDLE, "read_input: null argument");
  mlg_params_default(p);
  *run = mlg_run_params{};
  run->dt = 1.0e-3; run->ti = 0.0; run->totaltime = 1.0e2; run->ni = 0; run->totaln = 100000;   // mlegs_base.f90:17-25
  run->isfldsav = 1; run->fldsavintvl = 100; run->islogsav = 1; run->logsavintvl = 1;          // :43-51
  std::snprintf(run->flddir, sizeof run->flddir, "./output/fld/");
  std::snprintf(run->logdir, sizeof run->logdir, "./output/log/");
  FILE* f = std::fopen(fn, "r");
  if (!f) return set_error(MLG_EPARAM, "read_input: could not open input file");
  ListReader rd(f);
  std::string dum;
  std::vector<std::string> v;
  auto fail = [&](const char* msg) { std::fclose(f); return set_error(MLG_EPARAM, msg); };
  auto skip = [&]() { return rd.read1(&dum); };
  bool ok = true;
  // computational domain
  int xpi = 0;
  ok = ok && skip() && skip() && rd.read(&v, 3) && parse_int(v[0], &p->nr) && parse_int(v[1], &p->np) && parse_int(v[2], &p->nz);
  ok = ok && skip() && rd.read(&v, 3) && parse_int(v[0], &p->nrchop) && parse_int(v[1], &p->npchop) &&
       parse_int(v[2], &p->nzchop);
  ok = ok && skip() && rd.read(&v, 3) && parse_real(v[0], &p->ell) && parse_real(v[1], &p->zlen) && parse_logical(v[2], &xpi);
  if (ok && xpi) p->zlen *= 3.14159265358979323846;
  ok = ok && skip();
  // time stepping
  ok = ok && skip() && skip() && rd.read(&v, 5) && parse_real(v[0], &run->dt) && parse_real(v[1], &run->ti) &&
       parse_real(v[2], &run->totaltime) && parse_int(v[3], &run->ni) && parse_int(v[4], &run->totaln);
  ok = ok && skip();
  // flow field properties
  ok = ok && skip() && skip() && rd.read(&v, 3) && parse_real(v[0], &p->visc) && parse_int(v[1], &p->hyperpow) &&
       parse_real(v[2], &p->hypervisc);
  ok = ok && skip();
  if (!ok) return fail("read_input: could not read the domain, time-stepping and flow values");
  // data storage
  std::string line;
  if (!(skip() && skip() && rd.raw_line(&line))) return fail("read_input: could not read the field output directory");
  std::string fld = trim(line.substr(0, 256));
  if (fld.empty() || fld.back() != '/') fld += "/";
  if (!dir_ok(fld)) return fail("read_input: invalid field output directory");
  if (!(skip() && rd.read(&v, 2) && parse_logical(v[0], &run->isfldsav) && parse_int(v[1], &run->fldsavintvl) && skip()))
    return fail("read_input: could not read the field output settings");
  // data logging
  if (!(skip() && skip() && rd.raw_line(&line))) return fail("read_input: could not read the log output directory");
  std::string logd = trim(line.substr(0, 256));
  if (logd.empty() || logd.back() != '/') logd += "/";
  if (!dir_ok(logd)) return fail("read_input: invalid log output directory");
  if (!(skip() && rd.read(&v, 2) && parse_logical(v[0], &run->islogsav) && parse_int(v[1], &run->logsavintvl)))
    return fail("read_input: could not read the log output settings");
  // optional stability controls: older files end at the previous line
  if (skip() && skip()) {
    if (!(rd.read(&v, 5) && parse_logical(v[0], &p->is_svv) && parse_real(v[1], &p->svv_cutoff) &&
          parse_real(v[2], &p->svv_target) && parse_real(v[3], &p->svv_strength) && parse_real(v[4], &p->svv_relax)))
      return fail("read_input: invalid SVV controls");
  }
  std::fclose(f);
  if (fld.size() >= sizeof run->flddir || logd.size() >= sizeof run->logdir)
    return set_error(MLG_EPARAM, "read_input: output directory name too long");
  std::snprintf(run->flddir, sizeof run->flddir, "%s", fld.c_str());
  std::snprintf(run->logdir, sizeof run->logdir, "%s", logd.c_str());
  if (make_dirs) {
    if (mkdir_p(fld)) return set_error(MLG_EPARAM, "read_input: could not create field output directory");
    if (mkdir_p(logd)) return set_error(MLG_EPARAM, "read_input: could not create log output directory");
  }
  // the checks of :363-386
  if (p->nr <= 0 || p->nr % 2 != 0 || p->np <= 0 || p->nz <= 0)
    return set_error(MLG_EPARAM, "read_input: nr must be positive and even; np and nz must be positive");
  if (p->nrchop <= 0 || p->nrchop > p->nr || p->npchop <= 0 || p->npchop > p->np / 2 + 1 || p->nzchop <= 0 ||
      p->nzchop > p->nz / 2 + 1)
    return set_error(MLG_EPARAM, "read_input: invalid chopping sizes");
  if (p->ell <= 0.0 || p->zlen <= 0.0) return set_error(MLG_EPARAM, "read_input: ell and zlen must be positive");
  if (run->dt <= 0.0 || run->totaltime < 0.0 || run->totaln < 0)
    return set_error(MLG_EPARAM, "read_input: invalid time stepping values");
  if (p->visc < 0.0 || p->hypervisc < 0.0) return set_error(MLG_EPARAM, "read_input: viscosities must be non-negative");
  if (p->hyperpow != 0 && p->hyperpow != 4 && p->hyperpow != 6 && p->hyperpow != 8)
    return set_error(MLG_EPARAM, "read_input: hyperpow must be zero, 4, 6, or 8");
  if (p->hyperpow != 0 && p->hypervisc <= 0.0)
    return set_error(MLG_EPARAM, "read_input: hypervisc must be positive when enabled");
  if (run->fldsavintvl <= 0 || run->logsavintvl <= 0)
    return set_error(MLG_EPARAM, "read_input: output intervals must be positive");
  if (p->svv_cutoff <= 0.0 || p->svv_cutoff >= 1.0 || p->svv_target <= 0.0 || p->svv_strength < 0.0 ||
      p->svv_relax < 0.0 || p->svv_relax > 1.0)
    return set_error(MLG_EPARAM, "read_input: invalid SVV controls");
  return 0;
}

}  // extern "C"
