// Host side of the reference executable around the time step: the &namctl
// namelist (common/gocean2d_io_mod.f90:22-80), the single-rank model set-up
// (T mask of common/model_mod.f90:94-249, grid metrics and coordinates of
// original/nemolite2d.f90:218-290, initial state of
// common/initialisation_mod.f90:7-63), and the ASCII outputs the reference
// writes: go2d_<istp>_<rank>.dat (gocean2d_io_mod.f90:97-149) and
// tmask_<rank>.dat (model_mod.f90:251-291), byte for byte in the layout of
// the Fortran edit descriptors E16.7, I4 and I3.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/nl2d_gpu.h"

namespace {

// Fortran Ew.d output of one value (gfortran's form): [-]0.<d digits>E+ee,
// or [-]0.<d digits>+eee once the exponent needs three digits, right-
// justified in w columns; w asterisks if it does not fit.  The digits are
// the correctly rounded d significant digits of the binary value.
std::string fortran_e(double v, int w, int d) {
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
    if ((int)s.size() > w) s = v < 0 ? "-Inf" : "Inf";
  } else {
    const bool neg = std::signbit(v);
    const double a = std::fabs(v);
    std::string digits;
    int e10 = 0;
    if (a == 0.0) {
      digits.assign((size_t)d, '0');
    } else {
      // "%.*e" gives d significant digits as D.DDDDDDe+XX: value =
      // 0.DDDDDDD x 10^(XX + 1)
      char buf[64];
      std::snprintf(buf, sizeof buf, "%.*e", d - 1, a);
      const char* p = buf;
      digits.push_back(*p++);
      if (*p == '.') p++;
      while (*p && *p != 'e') digits.push_back(*p++);
      e10 = std::atoi(p + 1) + 1;
    }
    char ebuf[16];
    if (std::abs(e10) <= 99)
      std::snprintf(ebuf, sizeof ebuf, "E%c%02d", e10 < 0 ? '-' : '+', std::abs(e10));
    else
      std::snprintf(ebuf, sizeof ebuf, "%c%03d", e10 < 0 ? '-' : '+', std::abs(e10));
    s = std::string(neg ? "-" : "") + "0." + digits + ebuf;
  }
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

// Fortran Iw output: right-justified, w asterisks if it does not fit.
std::string fortran_i(long long v, int w) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%lld", v);
  const std::string s(buf);
  if ((int)s.size() > w) return std::string((size_t)w, '*');
  return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

std::string join_path(const char* dir, const std::string& name) {
  if (!dir || !*dir) return name;
  std::string p(dir);
  if (p.back() != '/') p.push_back('/');
  return p + name;
}

}  // namespace

extern "C" {

int nl2d_format_e(double v, int w, int d, char* out, int cap) {
  if (!out || w < 1 || d < 1 || cap < w + 1) return NL2D_ERR_ARGS;
  const std::string s = fortran_e(v, w, d);
  std::memcpy(out, s.c_str(), s.size() + 1);
  return NL2D_OK;
}

// The &namctl group: `key = value` items separated by commas, blanks or
// line ends, `!` comments, case-insensitive keys, Fortran real literals
// (1.5d-4), `/` closing the group; other groups before it are skipped, as a
// namelist READ skips them.  ints = (jpiglo, jpjglo, jphgr_msh, nit000,
// nitend, irecord), dbls = (dx, dy, dep_const, rdt, cbfr, visc); keys the
// file does not set keep the reference's defaults (gocean2d_io_mod.f90:57-68).
int nl2d_read_namelist(const char* path, int* ints, double* dbls) {
  static const char* const ikeys[6] = {"jpiglo", "jpjglo", "jphgr_msh",
                                       "nit000", "nitend", "irecord"};
  static const char* const dkeys[6] = {"dx", "dy", "dep_const", "rdt", "cbfr", "visc"};
  static const int idef[6] = {50, 100, 1, 1, 1000, 1};
  static const double ddef[6] = {1000.0, 1000.0, 100.0, 10.0, 0.001, 100.0};
  if (!path || !ints || !dbls) return NL2D_ERR_ARGS;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return NL2D_ERR_IO;
  std::string text;
  char chunk[4096];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, fp)) > 0) text.append(chunk, got);
  std::fclose(fp);
  // comments out, lower case
  std::string src;
  src.reserve(text.size());
  bool comment = false;
  for (char c : text) {
    if (c == '\n') comment = false;
    if (c == '!') comment = true;
    src.push_back(comment ? ' ' : (char)std::tolower((unsigned char)c));
  }
  for (int k = 0; k < 6; k++) {
    ints[k] = idef[k];
    dbls[k] = ddef[k];
  }
  size_t p = 0;
  const size_t n = src.size();
  auto skip_sep = [&]() {
    while (p < n && (std::isspace((unsigned char)src[p]) || src[p] == ',')) p++;
  };
  // find "&namctl" as a whole group name
  bool found = false;
  while (!found) {
    const size_t at = src.find("&namctl", p);
    if (at == std::string::npos) return NL2D_ERR_PARSE;
    const size_t after = at + 7;
    if (after >= n || !(std::isalnum((unsigned char)src[after]) || src[after] == '_')) {
      p = after;
      found = true;
    } else {
      p = after;
    }
  }
  for (;;) {
    skip_sep();
    if (p >= n) return NL2D_ERR_PARSE;  // the group never closed
    if (src[p] == '/') return NL2D_OK;
    if (src.compare(p, 4, "&end") == 0) return NL2D_OK;
    const size_t k0 = p;
    while (p < n && (std::isalnum((unsigned char)src[p]) || src[p] == '_')) p++;
    const std::string key = src.substr(k0, p - k0);
    if (key.empty()) return NL2D_ERR_PARSE;
    while (p < n && std::isspace((unsigned char)src[p])) p++;
    if (p >= n || src[p] != '=') return NL2D_ERR_PARSE;
    p++;
    while (p < n && std::isspace((unsigned char)src[p])) p++;
    const size_t v0 = p;
    while (p < n && !std::isspace((unsigned char)src[p]) && src[p] != ',' && src[p] != '/') p++;
    std::string val = src.substr(v0, p - v0);
    if (val.empty()) return NL2D_ERR_PARSE;
    int slot = -1;
    bool is_int = false;
    for (int k = 0; k < 6 && slot < 0; k++)
      if (key == ikeys[k]) slot = k, is_int = true;
    for (int k = 0; k < 6 && slot < 0; k++)
      if (key == dkeys[k]) slot = k;
    if (slot < 0) return NL2D_ERR_PARSE;  // not a member of namctl
    char* end = nullptr;
    if (is_int) {
      const long v = std::strtol(val.c_str(), &end, 10);
      if (*end != '\0') return NL2D_ERR_PARSE;
      ints[slot] = (int)v;
    } else {
      for (char& c : val)
        if (c == 'd') c = 'e';  // Fortran double-precision exponent
      const double v = std::strtod(val.c_str(), &end);
      if (*end != '\0') return NL2D_ERR_PARSE;
      dbls[slot] = v;
    }
  }
}

// Single-rank model set-up into caller-owned row-major [height][width]
// arrays (width >= jpiglo + 1, height >= jpjglo + 1; internal T cells
// 1..jpiglo-2 by 1..jpjglo-2, 0-based).  fields: the 13 field pointers in
// c_invoke_time_step's order; metrics: area_t, area_u, area_v, dx_u, dx_v,
// dx_t, dy_u, dy_v, dy_t, gphiu, gphiv; xt / yt may be NULL.
//  * T mask (model_mod.f90:144-239, one rank owning the whole domain): wet
//    inside, solid west and north, east open (-1) for jphgr_msh 2 and 3,
//    south open for 1 and 3, assigned in that order so the south row wins
//    the corners.  Columns and rows past the reference's jpiglo x jpjglo
//    mask follow the same rule.
//  * metrics: dx, dy, areas dx * dy, gphi 50 degrees everywhere
//    (original/nemolite2d.f90:218-232, 267-290).
//  * coordinates: xt = dx / 2 on the first internal column, then + dx per
//    column; yt likewise (original/nemolite2d.f90:236-246).
//  * state: depths dep_const, everything else zero; sshn_u / sshn_v of a
//    zero sshn_t are zero (initialisation_mod.f90:24-62).
//  * jphgr_msh = 0 (a STOP upstream: "read from a file" was never written)
//    keeps the caller's tmask as it is, e.g. one read by
//    nl2d_read_grid_file; everything else is set up as above.
int nl2d_setup_model(int jphgr_msh, int jpiglo, int jpjglo, double dx, double dy,
                     double dep_const, int width, int height, double* const* fields,
                     int* tmask, double* const* metrics, double* xt, double* yt) {
  if (jphgr_msh < 0 || jphgr_msh > 3 || jpiglo < 4 || jpjglo < 4 || width < jpiglo + 1 ||
      height < jpjglo + 1 || !fields || !tmask || !metrics)
    return NL2D_ERR_ARGS;
  for (int k = 0; k < 13; k++)
    if (!fields[k]) return NL2D_ERR_ARGS;
  for (int k = 0; k < 11; k++)
    if (!metrics[k]) return NL2D_ERR_ARGS;
  const int xs = 1, xe = jpiglo - 2, ys = 1, ye = jpjglo - 2;
  const size_t cells = (size_t)width * height;
  const bool east_open = jphgr_msh == 2 || jphgr_msh == 3;
  const bool south_open = jphgr_msh == 1 || jphgr_msh == 3;
  for (int j = 0; j < height && jphgr_msh != 0; j++)
    for (int i = 0; i < width; i++) {
      int m = (i >= xs && i <= xe && j >= ys && j <= ye) ? 1 : 0;
      if (i < xs) m = 0;
      if (j > ye) m = 0;
      if (i > xe) m = east_open ? -1 : 0;
      if (j < ys) m = south_open ? -1 : 0;
      tmask[(size_t)j * width + i] = m;
    }
  // fields in c_invoke_time_step order: ssha_t, sshn_t, sshn_u, sshn_v, hu,
  // hv, un, vn, ua, ht, ssha_u, va, ssha_v
  static const bool is_depth[13] = {false, false, false, false, true, true, false,
                                    false, false, true, false, false, false};
  for (int k = 0; k < 13; k++) {
    const double v = is_depth[k] ? dep_const : 0.0;
    for (size_t c = 0; c < cells; c++) fields[k][c] = v;
  }
  const double area = dx * dy;
  const double mval[11] = {area, area, area, dx, dx, dx, dy, dy, dy, 50.0, 50.0};
  for (int k = 0; k < 11; k++)
    for (size_t c = 0; c < cells; c++) metrics[k][c] = mval[k];
  if (xt || yt) {
    double* colx = (double*)std::malloc(sizeof(double) * (size_t)width);
    double* rowy = (double*)std::malloc(sizeof(double) * (size_t)height);
    if (!colx || !rowy) {
      std::free(colx);
      std::free(rowy);
      return NL2D_ERR_ARGS;
    }
    colx[xs] = 0.0 + 0.5 * dx;
    for (int i = xs + 1; i < width; i++) colx[i] = colx[i - 1] + dx;
    for (int i = xs - 1; i >= 0; i--) colx[i] = colx[i + 1] - dx;
    rowy[ys] = 0.0 + 0.5 * dy;
    for (int j = ys + 1; j < height; j++) rowy[j] = rowy[j - 1] + dy;
    for (int j = ys - 1; j >= 0; j--) rowy[j] = rowy[j + 1] - dy;
    for (int j = 0; j < height; j++)
      for (int i = 0; i < width; i++) {
        if (xt) xt[(size_t)j * width + i] = colx[i];
        if (yt) yt[(size_t)j * width + i] = rowy[j];
      }
    std::free(colx);
    std::free(rowy);
  }
  return NL2D_OK;
}

// A grid file: whitespace-separated triples "i j value" (1-based i in
// 1..nx, j in 1..ny), one per point of the nx x ny mask, in any order, blank
// lines ignored: the layout dump_tmask writes raw (model_mod.f90:268-274),
// so a dumped mask reads back.  is_int: int values into `out` (a T mask),
// else doubles (a depth).  Row-major [][width] output, 0-based.  Every point
// must appear exactly once.
int nl2d_read_grid_file(const char* path, int nx, int ny, int width, int is_int, void* out) {
  if (!path || !out || nx < 1 || ny < 1 || width < nx) return NL2D_ERR_ARGS;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return NL2D_ERR_IO;
  std::string seen((size_t)nx * ny, '\0');
  long long count = 0;
  int rc = NL2D_OK;
  for (;;) {
    long i, j;
    int got = std::fscanf(fp, "%ld %ld", &i, &j);
    if (got == EOF) break;
    if (got != 2 || i < 1 || i > nx || j < 1 || j > ny) {
      rc = NL2D_ERR_PARSE;
      break;
    }
    const size_t c = (size_t)(j - 1) * width + (size_t)(i - 1);
    const size_t key = (size_t)(j - 1) * nx + (size_t)(i - 1);
    if (seen[key]) {
      rc = NL2D_ERR_PARSE;
      break;
    }
    seen[key] = 1;
    if (is_int) {
      long v;
      if (std::fscanf(fp, "%ld", &v) != 1) {
        rc = NL2D_ERR_PARSE;
        break;
      }
      static_cast<int*>(out)[c] = (int)v;
    } else {
      double v;
      if (std::fscanf(fp, "%lf", &v) != 1) {
        rc = NL2D_ERR_PARSE;
        break;
      }
      static_cast<double*>(out)[c] = v;
    }
    count++;
  }
  std::fclose(fp);
  if (rc == NL2D_OK && count != (long long)nx * ny) rc = NL2D_ERR_PARSE;
  return rc;
}

// Face depths from T-point depths: hu = (ht(i) + ht(i+1)) / 2 on the east
// face, hv = (ht(j) + ht(j+1)) / 2 on the north face; the last column / row
// copies ht.  (The reference sets all three to dep_const; a depth read from a
// file needs face values and this is the plain average.)
int nl2d_face_depths(int width, int height, const double* ht, double* hu, double* hv) {
  if (!ht || !hu || !hv || width < 1 || height < 1) return NL2D_ERR_ARGS;
  for (int j = 0; j < height; j++)
    for (int i = 0; i < width; i++) {
      const size_t c = (size_t)j * width + i;
      hu[c] = i + 1 < width ? 0.5 * (ht[c] + ht[c + 1]) : ht[c];
      hv[c] = j + 1 < height ? 0.5 * (ht[c] + ht[c + width]) : ht[c];
    }
  return NL2D_OK;
}

// Fortran I5.5: five digits, zero-padded; asterisks past 99999.
static std::string i5_5(int v) {
  if (v < 0 || v > 99999) return "*****";
  char b[8];
  std::snprintf(b, sizeof b, "%05d", v);
  return b;
}

// go2d_<istp>_<rank>.dat (gocean2d_io_mod.f90:97-149): for each internal T
// row, for each internal T point, `(6e16.7)` of x, y, depth, ssh and the
// velocities averaged to the T point, 0.5 (un(i-1) + un(i)) and
// 0.5 (vn(j-1) + vn(j)); an empty record after each row.  Writes into `dir`
// (the current directory if NULL or empty).
int nl2d_model_write(const char* dir, int istp, int rank, int width, int xs, int xe, int ys,
                     int ye, const double* xt, const double* yt, const double* ht,
                     const double* sshn, const double* un, const double* vn) {
  if (!xt || !yt || !ht || !sshn || !un || !vn || width < 1 || xs < 1 || ys < 1 || xe < xs ||
      ye < ys || xe >= width)
    return NL2D_ERR_ARGS;
  const std::string path = join_path(dir, "go2d_" + i5_5(istp) + "_" + i5_5(rank) + ".dat");
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) return NL2D_ERR_IO;
  std::string line;
  for (int j = ys; j <= ye; j++) {
    for (int i = xs; i <= xe; i++) {
      const size_t c = (size_t)j * width + i;
      const double rtmp1 = 0.5 * (un[c - 1] + un[c]);
      const double rtmp2 = 0.5 * (vn[c - width] + vn[c]);
      line.clear();
      for (double v : {xt[c], yt[c], ht[c], sshn[c], rtmp1, rtmp2}) line += fortran_e(v, 16, 7);
      line.push_back('\n');
      std::fputs(line.c_str(), fp);
    }
    std::fputc('\n', fp);
  }
  return std::fclose(fp) == 0 ? NL2D_OK : NL2D_ERR_IO;
}

// tmask_<rank>.dat (model_mod.f90:251-291).  raw: every point of the
// nx x ny global mask, `(3(I4,1x))` of i, j (1-based) and the mask value
// (the trailing 1x writes nothing at the end of a record); otherwise the
// internal T points, `(2e16.7,1x,I3)` of x, y and the mask.  An empty record
// after each row.
int nl2d_dump_tmask(const char* dir, int rank, int raw, int width, int nx, int ny,
                    const int* tmask, int xs, int xe, int ys, int ye, const double* xt,
                    const double* yt) {
  if (!tmask || width < nx || nx < 1 || ny < 1) return NL2D_ERR_ARGS;
  if (!raw && (!xt || !yt || xs < 0 || ys < 0 || xe < xs || ye < ys || xe >= width))
    return NL2D_ERR_ARGS;
  const std::string path = join_path(dir, "tmask_" + i5_5(rank) + ".dat");
  FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) return NL2D_ERR_IO;
  std::string line;
  if (raw) {
    for (int jj = 1; jj <= ny; jj++) {
      for (int ji = 1; ji <= nx; ji++) {
        line = fortran_i(ji, 4) + " " + fortran_i(jj, 4) + " " +
               fortran_i(tmask[(size_t)(jj - 1) * width + (ji - 1)], 4) + "\n";
        std::fputs(line.c_str(), fp);
      }
      std::fputc('\n', fp);
    }
  } else {
    for (int j = ys; j <= ye; j++) {
      for (int i = xs; i <= xe; i++) {
        const size_t c = (size_t)j * width + i;
        line = fortran_e(xt[c], 16, 7) + fortran_e(yt[c], 16, 7) + " " +
               fortran_i(tmask[c], 3) + "\n";
        std::fputs(line.c_str(), fp);
      }
      std::fputc('\n', fp);
    }
  }
  return std::fclose(fp) == 0 ? NL2D_OK : NL2D_ERR_IO;
}

}  // extern "C"
