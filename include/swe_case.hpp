// swe_case.hpp — C++ host side of the reference's set-up around the step:
//
//   read_my_data           SOURCES/read_data.f90:35-100 (markers found by
//                          read_until, SOURCES/tools.f90:3-19)
//   load_mesh_free_format  SFEMaNS/FEMSUB_OBJET/prep_mesh.f90:759-1035 (P1,
//                          2D: unformatted .FEM records, first-touch node
//                          renumbering, boundary sides of the kept domains)
//   dirichlet_nodes        SFEMaNS/FEMSUB/dir_nodes.f90:243-292,495-511, as
//                          construct_mesh calls it (SOURCES/mesh.f90:20-36)
//   init_case, sol_anal    SOURCES/condlim.f90:92-245, 311-831 per type_test
//
// Arrays are in the reference layout: jj(3, me) and jjs(2, mes) 1-based,
// rr(2, np), column-major.  Errors (a missing marker, a corrupt file, a
// type_test the reference STOPs on) throw std::runtime_error.  Plain C++17,
// no CUDA: link swe_case.cpp.
#ifndef SWE_CASE_HPP
#define SWE_CASE_HPP

#include <string>
#include <vector>

namespace swe {

// the inputs record fields read_my_data fills
struct DataFile {
  std::string directory, file_name;
  int nb_dom = 0;
  std::vector<int> list_dom;
  int type_fe = 1;
  double Tfinal = 0.0, CFL = 0.0;
  std::string viscosity_type, viscous_type;
  bool if_alpha_limit = false, if_lumped = false;
  int type_test = 0;
  std::vector<int> h_Dir_list, ux_Dir_list, uy_Dir_list;   // the first nb_Dir_bdy values
  double mannings = 0.0, lambdaSGN = 0.0;
  double epsilon = 1.e-4;
};

DataFile read_my_data(const std::string& path);

struct FemMesh {
  int np = 0, me = 0, mes = 0;
  std::vector<int> jj, jjs, sides;
  std::vector<double> rr;
};

FemMesh load_mesh_free_format(const std::string& path, const std::vector<int>& list_dom);

// sorted unique nodes (1-based) of the boundary edges on the listed sides
std::vector<int> dirichlet_nodes(const FemMesh& m, const std::vector<int>& sides);

struct CaseInit {
  std::vector<double> bath;
  double gravity = 9.81, max_water_h = 1.0, htiny = 1.e-4;
  double t0 = 0.0;             // inputs%time after init (1 for type 4)
  double tfinal = 0.0;         // init's own final time (types 5 and 11)
  bool sets_tfinal = false;
};

CaseInit init_case(int type_test, const FemMesh& m, double epsilon = 1.e-4);

// sol_anal(k, rr, t) at n points rr(2, n) into out(n).  bath is the module
// array, read by position as the reference does (types 1, 2 and 8 at t = 0).
void sol_anal(int type_test, int k, int n, const double* rr, double t, const double* bath, double gravity,
              double htiny, double* out);

}  // namespace swe

#endif  // SWE_CASE_HPP
