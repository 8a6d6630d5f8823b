// nemolite2d_gb300: the reference executable's driver
// (manual_versions/psykal_cpp/nemolite2d.f90:1-121 with common/model_mod.f90
// model_init) around this library's c_invoke_time_step.  It reads the
// &namctl namelist, sets up the single-rank domain, writes tmask_00000.dat
// and go2d_<istp>_00000.dat every irecord steps (step 0 included) as the
// reference does, runs nit000..nitend, and prints the ua / va checksums in
// the reference's `('ua checksum = ', E16.8)` layout.
//
// usage: nemolite2d_gb300 [namelist-path [output-dir]]
//   (defaults: ./namelist, the current directory)
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/nl2d_gpu.h"

namespace {

// physical_params_mod.f90:9-15
constexpr double kPi = 3.1415926535897932;
constexpr double kG = 9.80665;
constexpr double kOmega = 7.292116e-05;
const double kD2r = kPi / 180.0;

int report(const char* what) {
  char msg[512];
  const int st = nl2d_last_error(msg, sizeof msg);
  if (st != NL2D_OK) {
    std::fprintf(stderr, "nemolite2d_gb300: %s failed (%d): %s\n", what, st, msg);
    return 1;
  }
  return 0;
}

// field_checksum: the sum of |x| over a field's internal region, in the
// reference's loop order (j outer, i inner).
double checksum(const std::vector<double>& f, int width, int x0, int x1, int y0, int y1) {
  double s = 0.0;
  for (int j = y0; j <= y1; j++)
    for (int i = x0; i <= x1; i++) s = s + std::fabs(f[(size_t)j * width + i]);
  return s;
}

}  // namespace

int main(int argc, char** argv) {
  const char* nml = argc > 1 ? argv[1] : "namelist";
  const char* outdir = argc > 2 ? argv[2] : "";
  int iv[6];
  double dv[6];
  int rc = nl2d_read_namelist(nml, iv, dv);
  if (rc == NL2D_ERR_IO) {
    std::fprintf(stderr, "cannot open namelist file %s\n", nml);
    return 1;
  }
  if (rc != NL2D_OK) {
    std::fprintf(stderr, "err found in reading namelist file\n");
    return 1;
  }
  const int jpiglo = iv[0], jpjglo = iv[1], jphgr_msh = iv[2];
  const int nit000 = iv[3], nitend = iv[4], irecord = iv[5];
  const double dx = dv[0], dy = dv[1], dep_const = dv[2], rdt = dv[3], cbfr = dv[4],
               visc = dv[5];
  std::printf("&NAMCTL\n JPIGLO=%d,\n JPJGLO=%d,\n JPHGR_MSH=%d,\n DX=%.17g,\n DY=%.17g,\n"
              " DEP_CONST=%.17g,\n NIT000=%d,\n NITEND=%d,\n IRECORD=%d,\n RDT=%.17g,\n"
              " CBFR=%.17g,\n VISC=%.17g,\n /\n",
              jpiglo, jpjglo, jphgr_msh, dx, dy, dep_const, nit000, nitend, irecord, rdt, cbfr,
              visc);
  if (irecord < 1) {
    std::fprintf(stderr, "irecord must be positive\n");
    return 1;
  }

  const int width = jpiglo + 1, height = jpjglo + 1;
  const size_t cells = (size_t)width * height;
  // c_invoke_time_step's field order: ssha_t, sshn_t, sshn_u, sshn_v, hu,
  // hv, un, vn, ua, ht, ssha_u, va, ssha_v
  enum { SSHA_T, SSHN_T, SSHN_U, SSHN_V, HU, HV, UN, VN, UA, HT, SSHA_U, VA, SSHA_V };
  std::vector<std::vector<double>> f(13, std::vector<double>(cells));
  std::vector<std::vector<double>> g(11, std::vector<double>(cells));
  std::vector<int> tmask(cells);
  std::vector<double> xt(cells), yt(cells);
  double* fp[13];
  double* gp[11];
  for (int k = 0; k < 13; k++) fp[k] = f[k].data();
  for (int k = 0; k < 11; k++) gp[k] = g[k].data();
  if (jphgr_msh == 0) {
    // The grid from files (a STOP in the reference): the T mask from
    // tmask_in.dat in dump_tmask's raw layout ("i j mask" for every point of
    // the jpiglo x jpjglo mask); points past it stay land.
    rc = nl2d_read_grid_file("tmask_in.dat", jpiglo, jpjglo, width, 1, tmask.data());
    if (rc != NL2D_OK) {
      std::fprintf(stderr, "jphgr_msh = 0 reads the T mask from tmask_in.dat: %s\n",
                   rc == NL2D_ERR_IO ? "file not found" : "not one \"i j mask\" per point");
      return 1;
    }
  }
  rc = nl2d_setup_model(jphgr_msh, jpiglo, jpjglo, dx, dy, dep_const, width, height, fp,
                        tmask.data(), gp, xt.data(), yt.data());
  if (rc == NL2D_OK && jphgr_msh == 0) {
    // optional T-point depths from depth_in.dat ("i j depth"); the column
    // and row past the mask copy their neighbours; face depths are averages
    std::vector<double> ht(cells, dep_const);
    const int drc = nl2d_read_grid_file("depth_in.dat", jpiglo, jpjglo, width, 0, ht.data());
    if (drc == NL2D_OK) {
      for (int j = 0; j < height; j++)
        for (int i = 0; i < width; i++) {
          const int si = i < jpiglo ? i : jpiglo - 1, sj = j < jpjglo ? j : jpjglo - 1;
          f[HT][(size_t)j * width + i] = ht[(size_t)sj * width + si];
        }
      nl2d_face_depths(width, height, f[HT].data(), f[HU].data(), f[HV].data());
    } else if (drc != NL2D_ERR_IO) {
      std::fprintf(stderr, "depth_in.dat is not one \"i j depth\" per point\n");
      return 1;
    }
  }
  if (rc != NL2D_OK) {
    std::fprintf(stderr, "Wrong grid definition type (jphgr_msh must be 0, 1, 2 or 3), "
                         "check your namelist file.\n");
    return 1;
  }
  const int xs = 1, xe = jpiglo - 2, ys = 1, ye = jpjglo - 2;
  if (nl2d_dump_tmask(outdir, 0, 1, width, jpiglo, jpjglo, tmask.data(), xs, xe, ys, ye,
                      xt.data(), yt.data()) != NL2D_OK ||
      nl2d_model_write(outdir, 0, 0, width, xs, xe, ys, ye, xt.data(), yt.data(),
                       f[HT].data(), f[SSHN_T].data(), f[UN].data(),
                       f[VN].data()) != NL2D_OK) {
    std::fprintf(stderr, "cannot write the output files\n");
    return 1;
  }
  std::printf("Simulation domain = (%4d:%4d,%4d:%4d)\n", xs + 1, xe + 1, ys + 1, ye + 1);

  // time_step_mod.f90:65-79 passes dx_v and dx_t for dy_v and dy_t
  auto step = [&](int istp) {
    c_invoke_time_step(fp[SSHA_T], fp[SSHN_T], fp[SSHN_U], fp[SSHN_V], fp[HU], fp[HV], fp[UN],
                       fp[VN], fp[UA], fp[HT], fp[SSHA_U], fp[VA], fp[SSHA_V], tmask.data(),
                       gp[0], gp[1], gp[2], gp[3], gp[4], gp[5], gp[6], gp[4], gp[5], gp[9],
                       gp[10], istp, xs, xe, ys, ye, width, height, rdt, cbfr, visc, kOmega,
                       kD2r, kG);
  };
  auto read_back = [&](int k) {
    c_read_from_device(fp[k], fp[k], 1, 1, width, height, true);
  };

  const auto t0 = std::chrono::steady_clock::now();
  double write_s = 0.0;
  for (int istp = nit000; istp <= nitend; istp++) {
    step(istp);
    if (istp % irecord == 0) {
      const auto w0 = std::chrono::steady_clock::now();
      read_back(SSHN_T);
      read_back(UN);
      read_back(VN);
      if (report("step")) return 1;
      if (nl2d_model_write(outdir, istp, 0, width, xs, xe, ys, ye, xt.data(), yt.data(),
                           f[HT].data(), f[SSHN_T].data(), f[UN].data(),
                           f[VN].data()) != NL2D_OK) {
        std::fprintf(stderr, "cannot write go2d output for step %d\n", istp);
        return 1;
      }
      write_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    }
  }
  nl2d_sync();
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  read_back(UA);
  read_back(VA);
  if (report("time stepping")) return 1;

  char buf[32];
  // u internal region i in [xs, xe-1], j in [ys, ye]; v: i in [xs, xe], j in [ys, ye-1]
  nl2d_format_e(checksum(f[UA], width, xs, xe - 1, ys, ye), 16, 8, buf, sizeof buf);
  std::printf("ua checksum = %s\n", buf);
  nl2d_format_e(checksum(f[VA], width, xs, xe, ys, ye - 1), 16, 8, buf, sizeof buf);
  std::printf("va checksum = %s\n", buf);
  const long long nsteps = nitend >= nit000 ? (long long)(nitend - nit000 + 1) : 0;
  const double mcs = secs > 0 ? (double)(xe - xs + 1) * (ye - ys + 1) * nsteps / secs / 1e6 : 0;
  std::printf("Time-stepping: %lld steps in %.6f s (%.6f s writing output), %.1f Mcell-steps/s\n",
              nsteps, secs, write_s, mcs);
  nl2d_finalize();
  std::printf("Simulation finished!!\n");
  return 0;
}
