// swe_main: the reference's main program (SOURCES/main.f90) for the unit
// square dam break, written against the C++ host interface (swe_update.hpp)
// instead of the Fortran modules: mesh, init, construct_matrices, then
// DO WHILE(time < Tfinal) { COMPUTE_DT; three SSP-RK stages; bdy } on the
// device, with the time loop's VTK movie frames (main.f90:119-143).
//
//   swe_main [--n N] [--tfinal T] [--precision 0|1] [--frames K --dir D]
//            [--out state.bin]
//
// Mesh: N x N vertices on [0,1]^2, every cell cut along its SW->NE diagonal,
// vertices numbered x fastest; walls qx = 0 on x = 0, 1 and qy = 0 on
// y = 0, 1 (Dirichlet, as bdy imposes); h = 1 for x < 0.5, 0.1 elsewhere,
// q = 0.  Prints the steps, the final time and dt and the water mass; --out
// writes the final un(3, np) as raw FP64 (column-major).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swe_update.hpp"

namespace {

struct Mesh {
  int np = 0, me = 0;
  std::vector<int> jj;       // (3, me), 1-based
  std::vector<double> rr;    // (2, np)
};

// numpy.linspace(a, b, n)[i]: i * ((b - a) / (n - 1)) + a, the last point b
double lin(double a, double b, int n, int i) { return i == n - 1 ? b : i * ((b - a) / (n - 1)) + a; }

Mesh lattice(int n) {
  Mesh m;
  m.np = n * n;
  m.me = 2 * (n - 1) * (n - 1);
  m.rr.resize(2 * (size_t)m.np);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      m.rr[2 * (size_t)(i + n * j)] = lin(0.0, 1.0, n, i);
      m.rr[2 * (size_t)(i + n * j) + 1] = lin(0.0, 1.0, n, j);
    }
  for (int j = 0; j < n - 1; j++)
    for (int i = 0; i < n - 1; i++) {
      const int sw = i + n * j + 1, se = sw + 1, nw = sw + n, ne = sw + n + 1;
      const int t[6] = {sw, se, ne, sw, ne, nw};
      m.jj.insert(m.jj.end(), t, t + 6);
    }
  return m;
}

}  // namespace

int main(int argc, char** argv) {
  int n = 101, precision = SWE_PREC_FP64, nb_frame = 0;
  double tfinal = 0.2;
  std::string out, dir = ".";
  for (int a = 1; a + 1 < argc; a += 2) {
    const std::string k = argv[a];
    if (k == "--n") n = std::atoi(argv[a + 1]);
    else if (k == "--tfinal") tfinal = std::atof(argv[a + 1]);
    else if (k == "--precision") precision = std::atoi(argv[a + 1]);
    else if (k == "--frames") nb_frame = std::atoi(argv[a + 1]);
    else if (k == "--dir") dir = argv[a + 1];
    else if (k == "--out") out = argv[a + 1];
    else { std::fprintf(stderr, "unknown option %s\n", k.c_str()); return 2; }
  }
  if (n < 3 || !(tfinal > 0)) { std::fprintf(stderr, "need --n >= 3 and --tfinal > 0\n"); return 2; }
  const Mesh mesh = lattice(n);
  swe_params p{};
  p.gravity = 9.81; p.cfl = 0.25; p.max_water_h = 1.0; p.htiny = 1e-4 * p.max_water_h;
  p.type_test = 4; p.syst_size = 3; p.viscosity_type = SWE_VISC_FCT; p.viscous_type = 2;
  p.if_alpha_limit = 1; p.if_lumped = 1; p.if_roundoff_fix = 1; p.precision = precision;
  std::vector<double> bath(mesh.np, 0.0), un(3 * (size_t)mesh.np, 0.0);
  std::vector<int> jx, jy;
  for (int v = 0; v < mesh.np; v++) {
    const int i = v % n, j = v / n;
    un[3 * (size_t)v] = mesh.rr[2 * (size_t)v] < 0.5 ? 1.0 : 0.1;
    if (i == 0 || i == n - 1) jx.push_back(v + 1);
    if (j == 0 || j == n - 1) jy.push_back(v + 1);
  }
  try {
    swe::Update upd(mesh.np, mesh.me, mesh.jj.data(), mesh.rr.data(), bath.data(), p);
    upd.set_dirichlet(1, jx, std::vector<double>(jx.size(), 0.0));
    upd.set_dirichlet(2, jy, std::vector<double>(jy.size(), 0.0));
    double hmax0 = 0.0;
    for (int v = 0; v < mesh.np; v++) hmax0 = un[3 * (size_t)v] > hmax0 ? un[3 * (size_t)v] : hmax0;
    double time = 0.0, dt = 0.0;
    int steps = 0;
    if (nb_frame < 2) {                                          // the loop on the device, 64 steps a call
      for (;;) {
        double t = time;
        const int done = upd.rk3(un.data(), t, tfinal, 64, &dt);
        time = t;
        steps += done;
        if (done < 64) break;                                    // time reached Tfinal
      }
    } else {                                                     // a step at a time, with frames
      const double dt_frame = tfinal / (nb_frame - 1);
      double t_frame = 0.0;
      int kit = 0;
      if (swe_upload(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "upload");
      const double t0 = 0.0;
      if (swe_set_time(upd.context(), &t0, &tfinal) != SWE_OK) throw swe::Stop(SWE_ERR_ARG, "set_time");
      while (time < tfinal) {
        int done = 0;
        const int rc = swe_rk3_steps(upd.context(), 1, &time, &dt, &done);
        if (rc != SWE_OK) throw swe::Stop(rc, swe_last_error(upd.context()));
        if (!done) break;
        steps += done;
        if (time >= t_frame - 1.e-10) {                          // main.f90:122-143
          kit++;
          t_frame += dt_frame;
          const std::string k = std::to_string(kit);
          const std::string a = dir + "/hpz_" + k + ".vtk", b = dir + "/h_" + k + ".vtk";
          const int fr = swe_frame_async(upd.context(), 0, hmax0, a.c_str(), b.c_str());
          if (fr != SWE_OK) throw swe::Stop(fr, swe_last_error(upd.context()));
        }
      }
      const int fw = swe_frames_wait(upd.context());
      if (fw != SWE_OK) throw swe::Stop(fw, swe_last_error(upd.context()));
      if (swe_download(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "download");
    }
    std::printf("steps %d time %.17g dt %.17g mass %.17g\n", steps, time, dt, upd.total_mass());
    if (!out.empty()) {
      FILE* f = std::fopen(out.c_str(), "wb");
      if (!f || std::fwrite(un.data(), sizeof(double), un.size(), f) != un.size()) {
        std::fprintf(stderr, "cannot write %s\n", out.c_str());
        if (f) std::fclose(f);
        return 1;
      }
      std::fclose(f);
    }
  } catch (const swe::Stop& e) {   // the reference's WRITE + STOP
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
