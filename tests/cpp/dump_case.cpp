// Test tool for the C++ set-up (include/swe_case.hpp): prints what
// read_my_data, load_mesh_free_format, dirichlet_nodes, init_case and
// sol_anal give for a data file and a mesh, one "key values..." line each
// (reals as %.17g), for the Python host side to compare.  No CUDA.
//
//   dump_case DATA MESH [TYPE_TEST]     (TYPE_TEST overrides the data file's)
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "swe_case.hpp"

static void ints(const char* key, const std::vector<int>& v) {
  std::printf("%s", key);
  for (int x : v) std::printf(" %d", x);
  std::printf("\n");
}

static void reals(const char* key, const std::vector<double>& v) {
  std::printf("%s", key);
  for (double x : v) std::printf(" %.17g", x);
  std::printf("\n");
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    const swe::DataFile d = swe::read_my_data(argv[1]);
    std::printf("strings %s|%s|%s|%s\n", d.directory.c_str(), d.file_name.c_str(), d.viscosity_type.c_str(),
                d.viscous_type.c_str());
    std::printf("scalars %d %d %.17g %.17g %d %d %d %.17g %.17g\n", d.nb_dom, d.type_fe, d.Tfinal, d.CFL,
                (int)d.if_alpha_limit, (int)d.if_lumped, d.type_test, d.mannings, d.lambdaSGN);
    ints("list_dom", d.list_dom);
    ints("h_dir", d.h_Dir_list);
    ints("ux_dir", d.ux_Dir_list);
    ints("uy_dir", d.uy_Dir_list);
    const swe::FemMesh m = swe::load_mesh_free_format(argv[2], d.list_dom);
    ints("jj", m.jj);
    ints("jjs", m.jjs);
    ints("sides", m.sides);
    reals("rr", m.rr);
    ints("h_js", swe::dirichlet_nodes(m, d.h_Dir_list));
    ints("ux_js", swe::dirichlet_nodes(m, d.ux_Dir_list));
    ints("uy_js", swe::dirichlet_nodes(m, d.uy_Dir_list));
    const int tt = argc > 3 ? std::atoi(argv[3]) : d.type_test;
    const swe::CaseInit ci = swe::init_case(tt, m, d.epsilon);
    reals("bath", ci.bath);
    std::printf("init %.17g %.17g %.17g %.17g %.17g %d\n", ci.gravity, ci.max_water_h, ci.htiny, ci.t0, ci.tfinal,
                (int)ci.sets_tfinal);
    const int S = tt == 13 ? 5 : 3;
    std::vector<double> v(m.np);
    for (int k = 1; k <= S; k++) {
      swe::sol_anal(tt, k, m.np, m.rr.data(), ci.t0, ci.bath.data(), ci.gravity, ci.htiny, v.data());
      reals(("u0_" + std::to_string(k)).c_str(), v);
    }
    for (int k = 1; k <= 3; k++) {
      swe::sol_anal(tt, k, m.np, m.rr.data(), ci.t0 + 0.75, ci.bath.data(), ci.gravity, ci.htiny, v.data());
      reals(("sol_" + std::to_string(k)).c_str(), v);
    }
  } catch (const std::runtime_error& e) {
    std::printf("error %s\n", e.what());
    return 1;
  }
  return 0;
}
