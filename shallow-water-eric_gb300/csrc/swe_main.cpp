// swe_main: the reference's main program (SOURCES/main.f90) written against
// the C++ host interfaces (swe_update.hpp, swe_case.hpp) instead of the
// Fortran modules.  Two modes:
//
//   swe_main --data FILE [--mesh FILE] [--steps K] [--precision 0|1]
//            [--frames K --dir D] [--out state.bin]
//     main.f90:19-91 for a reference data file: read_my_data,
//     construct_mesh (the .FEM file named in it, relative to the data file's
//     directory, or --mesh), construct_matrices, init, then
//     DO WHILE(time < Tfinal) { COMPUTE_DT; three SSP-RK stages; bdy }, at
//     most K steps.  Where the values bdy writes stay fixed over
//     (t0, Tfinal] the loop runs on the device; where they change with time
//     it runs here over the per-call euler / compute_dij, with bdy at the
//     reference's stage times.  The loop's movie frames are written as
//     main.f90 writes them (nb_frame = 200 unless --frames says otherwise;
//     --frames 0 writes none), and compute_errors' relative L1 / L2 errors
//     on h are printed for the types that have an exact solution; types 1
//     and 2 write the loop's monitor to fort.10.
//
//   swe_main [--n N] [--tfinal T] [--precision 0|1] [--frames K --dir D]
//            [--out state.bin]
//     the unit-square dam break: N x N vertices on [0,1]^2, every cell cut
//     along its SW->NE diagonal, vertices numbered x fastest; walls qx = 0
//     on x = 0, 1 and qy = 0 on y = 0, 1 (Dirichlet, as bdy imposes); h = 1
//     for x < 0.5, 0.1 elsewhere, q = 0; on the device, with the time loop's
//     VTK movie frames (main.f90:119-143).
//
// Prints the steps, the final time and dt and the water mass; --out writes
// the final un(S, np) as raw FP64 (column-major).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/swe_case.hpp"
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

bool write_state(const std::string& out, const std::vector<double>& un) {
  if (out.empty()) return true;
  FILE* f = std::fopen(out.c_str(), "wb");
  if (!f || std::fwrite(un.data(), sizeof(double), un.size(), f) != un.size()) {
    std::fprintf(stderr, "cannot write %s\n", out.c_str());
    if (f) std::fclose(f);
    return false;
  }
  std::fclose(f);
  return true;
}

// main.f90:19-91 for a data file (see the header comment)
int run_data(const std::string& data_path, std::string mesh_path, int max_steps, int precision,
             const std::string& out, int nb_frame, const std::string& dir) {
  const swe::DataFile d = swe::read_my_data(data_path);
  if (mesh_path.empty()) {
    const size_t slash = data_path.find_last_of('/');
    const std::string base = slash == std::string::npos ? "." : data_path.substr(0, slash);
    mesh_path = base + "/" + d.directory + "/" + d.file_name;
  }
  const swe::FemMesh m = swe::load_mesh_free_format(mesh_path, d.list_dom);
  const int tt = d.type_test, S = tt == 13 ? 5 : 3;
  const swe::CaseInit ci = swe::init_case(tt, m, d.epsilon);
  std::string visc = d.viscosity_type;
  while (!visc.empty() && visc.back() == ' ') visc.pop_back();
  swe_params p{};
  p.gravity = ci.gravity; p.cfl = d.CFL; p.htiny = ci.htiny; p.mannings = d.mannings;
  p.lambda_sgn = d.lambdaSGN; p.max_water_h = ci.max_water_h; p.type_test = tt; p.syst_size = S;
  p.viscosity_type = visc == "galerkin" ? SWE_VISC_GALERKIN : visc == "viscous" ? SWE_VISC_VISCOUS
                   : visc == "entropy_visc" ? SWE_VISC_ENTROPY : visc == "fct" ? SWE_VISC_FCT : -1;
  if (p.viscosity_type < 0) throw swe::Stop(SWE_ERR_ARG, "viscosity type '" + visc + "'");
  if (d.viscous_type != "type1" && d.viscous_type != "type2")
    throw swe::Stop(SWE_ERR_ARG, "first-order viscosity '" + d.viscous_type + "'");
  p.viscous_type = d.viscous_type == "type1" ? 1 : 2;
  p.if_alpha_limit = d.if_alpha_limit; p.if_lumped = d.if_lumped; p.if_roundoff_fix = 1;
  p.precision = precision;
  const double t0 = ci.t0, tfinal = ci.sets_tfinal ? ci.tfinal : d.Tfinal;
  // un(k,:) = sol_anal(k, rr, time) (condlim.f90:235-237)
  std::vector<double> un((size_t)S * m.np), col(m.np);
  for (int k = 1; k <= S; k++) {
    swe::sol_anal(tt, k, m.np, m.rr.data(), t0, ci.bath.data(), ci.gravity, ci.htiny, col.data());
    for (int i = 0; i < m.np; i++) un[(size_t)S * i + k - 1] = col[i];
  }
  // bdy (main.f90:176-188): h on h_js_D, qx on ux_js_D, qy on uy_js_D, and
  // for type 13 the fourth and fifth unknowns on ux_js_D and uy_js_D
  struct Bc { int comp; std::vector<int> js; std::vector<double> rr, val; };
  std::vector<Bc> bcs;
  const std::vector<int>* lists[3] = {&d.h_Dir_list, &d.ux_Dir_list, &d.uy_Dir_list};
  for (int c = 0; c < (tt == 13 ? 5 : 3); c++) {
    Bc b;
    b.comp = c;
    b.js = swe::dirichlet_nodes(m, *lists[c < 3 ? c : c - 2]);
    if (b.js.empty()) continue;
    for (int j : b.js) { b.rr.push_back(m.rr[2 * (size_t)(j - 1)]); b.rr.push_back(m.rr[2 * (size_t)(j - 1) + 1]); }
    b.val.resize(b.js.size());
    bcs.push_back(b);
  }
  auto bdy_values = [&](Bc& b, double t) {
    swe::sol_anal(tt, b.comp + 1, (int)b.js.size(), b.rr.data(), t, ci.bath.data(), ci.gravity, ci.htiny,
                  b.val.data());
  };
  // fixed over (t0, Tfinal]? the values at t0 + 1e-6 and at 16 times up to Tfinal
  bool fixed = true;
  for (Bc& b : bcs) {
    std::vector<double> first;
    for (int s = 0; s <= 16 && fixed; s++) {
      const double t = s == 0 ? t0 + 1.e-6 : lin(t0, tfinal, 17, s);
      try {
        bdy_values(b, t);
      } catch (const std::runtime_error&) {
        fixed = false;
        break;
      }
      if (s == 0) first = b.val;
      else if (b.val != first) fixed = false;
    }
  }
  swe::Update upd(m.np, m.me, m.jj.data(), m.rr.data(), ci.bath.data(), p);
  double time = t0, dt = 0.0;
  int steps = 0;
  // movie frames (main.f90:42-47, 119-143): types 5, 8, 9, 11, 12, 13 every
  // Tfinal/(nb_frame-1), starting with the first step; type 3 writes frames
  // too but never sets dt_frame (zero): a frame after every step
  const bool frame_type = tt == 5 || tt == 8 || tt == 9 || tt == 11 || tt == 12 || tt == 13;
  const bool movie = nb_frame > 1 && (frame_type || tt == 3);
  double hmax0 = 0.0;
  for (int i = 0; i < m.np; i++) hmax0 = std::max(hmax0, un[(size_t)S * i]);
  double dt_frame = 0.0, t_frame = 0.0;
  int kit = 0;
  auto vtk = [&](const std::string& name, const std::string& title, const std::vector<double>& f) {
    const std::string path = dir + "/" + name;
    if (swe_write_vtk_2d(path.c_str(), title.c_str(), m.np, m.me, m.jj.data(), m.rr.data(), f.data()) != SWE_OK)
      throw swe::Stop(SWE_ERR_ARG, "cannot write " + path);
  };
  if (movie && frame_type) {
    dt_frame = tfinal / (nb_frame - 1);
    vtk("bath.vtk", "bath.vtk", ci.bath);
    std::vector<double> hex(m.np);
    swe::sol_anal(tt, 1, m.np, m.rr.data(), tfinal, ci.bath.data(), ci.gravity, ci.htiny, hex.data());
    vtk("hexact.vtk", "hexact.vtk", hex);
  }
  auto frame_due = [&]() {
    if (!movie || !(0.0 <= time) || !(time >= t_frame - 1.e-10)) return std::string();
    kit++;
    t_frame += dt_frame;
    return kit < 1000 ? std::to_string(kit) : std::string("***");   // WRITE(frame,'(I3)') kit
  };
  // the monitor of main.f90:94-99 for types 1 and 2: time and
  // 0.5 (|qx|_1 + |qy|_1) / (g |h^(3/2)|_1) after every step, into fort.10
  // (the unit it WRITEs to), from the device state
  FILE* mon = nullptr;
  if (tt == 1 || tt == 2) {
    const std::string path = dir + "/fort.10";
    mon = std::fopen(path.c_str(), "w");
    if (!mon) throw swe::Stop(SWE_ERR_ARG, "cannot write " + path);
  }
  auto monitor = [&]() {
    if (!mon) return;
    double q1 = 0.0, q2 = 0.0, q3 = 0.0;
    if (swe_norms(upd.context(), 0, 1, nullptr, &q1, nullptr) != SWE_OK ||
        swe_norms(upd.context(), 0, 2, nullptr, &q2, nullptr) != SWE_OK ||
        swe_norms(upd.context(), 0, SWE_FIELD_H32, nullptr, &q3, nullptr) != SWE_OK)
      throw swe::Stop(SWE_ERR_CUDA, swe_last_error(upd.context()));
    std::fprintf(mon, "%.17g %.17g\n", time, 0.5 * (q1 + q2) / (ci.gravity * q3));
  };
  if (fixed) {
    for (Bc& b : bcs) upd.set_dirichlet(b.comp, b.js, b.val);
  }
  if (fixed && (movie || mon)) {                                 // a step at a time: frames, monitor
    if (swe_upload(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "upload");
    if (swe_set_time(upd.context(), &time, &tfinal) != SWE_OK) throw swe::Stop(SWE_ERR_ARG, "set_time");
    while (time < tfinal && steps < max_steps) {
      int done = 0;
      const int rc = swe_rk3_steps(upd.context(), 1, &time, &dt, &done);
      if (rc != SWE_OK) throw swe::Stop(rc, swe_last_error(upd.context()));
      if (!done) break;
      steps += done;
      monitor();
      const std::string k = frame_due();
      if (!k.empty()) {
        const std::string a = dir + "/hpz_" + k + ".vtk", b = dir + "/h_" + k + ".vtk";
        const int fr = swe_frame_async(upd.context(), 0, hmax0, a.c_str(), b.c_str());
        if (fr != SWE_OK) throw swe::Stop(fr, swe_last_error(upd.context()));
      }
    }
    const int fw = swe_frames_wait(upd.context());
    if (fw != SWE_OK) throw swe::Stop(fw, swe_last_error(upd.context()));
    if (swe_download(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "download");
  } else if (fixed) {
    while (steps < max_steps) {
      const int chunk = std::min(64, max_steps - steps);
      double t = time;
      const int done = upd.rk3(un.data(), t, tfinal, chunk, &dt);
      time = t;
      steps += done;
      if (done < chunk) break;
    }
  } else {                                                       // main.f90:61-91 over the per-call ABI
    auto bdy = [&](std::vector<double>& uu, double t) {
      for (Bc& b : bcs) {
        bdy_values(b, t);
        for (size_t q = 0; q < b.js.size(); q++) uu[(size_t)S * (b.js[q] - 1) + b.comp] = b.val[q];
      }
    };
    std::vector<double> uo, ui(un.size()), dij(upd.nnz());
    while (time < tfinal && steps < max_steps) {
      dt = upd.compute_dij(un.data(), dij.data());               // COMPUTE_DT
      p.dt = dt;
      upd.set_inputs(p);
      const double to = time;
      uo = un;
      upd.euler(uo.data(), un.data());
      bdy(un, time + dt);
      time = to + dt;
      upd.euler(un.data(), ui.data());
      for (size_t q = 0; q < un.size(); q++) un[q] = (3 * uo[q] + ui[q]) / 4;
      bdy(un, time + dt / 2);
      time = to + dt / 2;
      upd.euler(un.data(), ui.data());
      for (size_t q = 0; q < un.size(); q++) un[q] = (uo[q] + 2 * ui[q]) / 3;
      bdy(un, time + dt);
      time = to + dt;
      steps++;
      if (mon) {
        if (swe_upload(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "upload");
        monitor();
      }
      const std::string k = frame_due();
      if (!k.empty()) {                                          // the frame fields of main.f90:124-141
        std::vector<double> hpz(m.np), h(m.np);
        for (int i = 0; i < m.np; i++) {
          const double hi = un[(size_t)S * i];
          const bool dry = hi <= 1.e-4 * hmax0;
          hpz[i] = dry ? -1.e-7 * hmax0 + ci.bath[i] : hi + ci.bath[i];
          h[i] = dry ? 0.0 : hi;
        }
        const std::string a = "hpz_" + k + ".vtk", b = "h_" + k + ".vtk";
        vtk(a, std::string(a).append(200 - a.size(), ' '), hpz);
        vtk(b, std::string(b).append(200 - b.size(), ' '), h);
      }
    }
    if (swe_upload(upd.context(), un.data()) != SWE_OK) throw swe::Stop(SWE_ERR_CUDA, "upload");
  }
  if (mon) std::fclose(mon);
  std::printf("type %d np %d %s steps %d time %.17g dt %.17g mass %.17g\n", tt, m.np,
              fixed ? "device-loop" : "per-call", steps, time, dt, upd.total_mass());
  // compute_errors (main.f90:198-263): relative L1 and L2 errors on h at the
  // Gauss points against sol_anal(1, r_gauss, time), on the device state
  if (tt == 3 || tt == 4 || tt == 5 || tt == 6 || tt == 7 || tt == 11 || tt == 12 || tt == 13) {
    std::vector<double> rj(3 * (size_t)m.me), rg(6 * (size_t)m.me), fa(3 * (size_t)m.me);
    if (swe_gauss_points(upd.context(), 0, rj.data(), rg.data()) != SWE_OK)
      throw swe::Stop(SWE_ERR_CUDA, swe_last_error(upd.context()));
    swe::sol_anal(tt, 1, 3 * m.me, rg.data(), time, ci.bath.data(), ci.gravity, ci.htiny, fa.data());
    double e1 = 0.0, e2 = 0.0, n1 = 0.0, n2 = 0.0;
    if (swe_norms(upd.context(), 0, 0, fa.data(), &e1, &e2) != SWE_OK)
      throw swe::Stop(SWE_ERR_CUDA, swe_last_error(upd.context()));
    for (size_t q = 0; q < fa.size(); q++) { n1 += std::fabs(fa[q]) * rj[q]; n2 += fa[q] * fa[q] * rj[q]; }
    n2 = std::sqrt(n2);
    std::printf(" Total number of elements %d\n Total number of points   %d\n", m.me, m.np);
    std::printf(" Relative L1 error on h (Gaussian) %.17g\n Relative L2 error on h (Gaussian) %.17g\n", e1 / n1,
                e2 / n2);
  }
  return write_state(out, un) ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
  int n = 101, precision = SWE_PREC_FP64, nb_frame = 0, max_steps = 1 << 30;
  bool nb_frame_set = false;
  double tfinal = 0.2;
  std::string out, dir = ".", data, mesh_file;
  for (int a = 1; a + 1 < argc; a += 2) {
    const std::string k = argv[a];
    if (k == "--n") n = std::atoi(argv[a + 1]);
    else if (k == "--tfinal") tfinal = std::atof(argv[a + 1]);
    else if (k == "--precision") precision = std::atoi(argv[a + 1]);
    else if (k == "--frames") { nb_frame = std::atoi(argv[a + 1]); nb_frame_set = true; }
    else if (k == "--dir") dir = argv[a + 1];
    else if (k == "--out") out = argv[a + 1];
    else if (k == "--data") data = argv[a + 1];
    else if (k == "--mesh") mesh_file = argv[a + 1];
    else if (k == "--steps") max_steps = std::atoi(argv[a + 1]);
    else { std::fprintf(stderr, "unknown option %s\n", k.c_str()); return 2; }
  }
  if (!data.empty()) {
    try {
      return run_data(data, mesh_file, max_steps, precision, out, nb_frame_set ? nb_frame : 200, dir);
    } catch (const swe::Stop& e) {   // the reference's WRITE + STOP
      std::fprintf(stderr, "%s\n", e.what());
      return 3;
    } catch (const std::runtime_error& e) {
      std::fprintf(stderr, "%s\n", e.what());
      return 2;
    }
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
    if (!write_state(out, un)) return 1;
  } catch (const swe::Stop& e) {   // the reference's WRITE + STOP
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}
