// Legacy-VTK writer of P1 fields, byte for byte the text of the reference's
// vtk_2d (SFEMaNS/FEMSUB/sub_plot.f90:1036-1095, P1 branch :1063-1071): the
// Fortran edit descriptors E13.7, I7, I8, 2X and 1X are restated here
// (gfortran conventions: a negative E13.7 drops the optional leading zero,
// a positional X at the end of a record writes nothing, an integer too wide
// for its field prints asterisks).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/swe_gpu.h"
#include "swe_setup.hpp"

#define SWE_API extern "C" __attribute__((visibility("default")))

namespace {

// Fortran Ew.d with w = 13, d = 7: "0.dddddddE+xx" (mantissa in [0.1, 1)),
// "-.dddddddE+xx" for negative values, "0.ddddddd+xxx" for 3-digit exponents.
void put_e13_7(std::string& out, double x) {
  if (std::isnan(x)) { out += "          NaN"; return; }
  if (std::isinf(x)) { out += x > 0 ? "     Infinity" : "    -Infinity"; return; }
  const bool neg = std::signbit(x);
  char digits[8] = "0000000";
  int exp10 = 0;
  if (x != 0.0) {
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.6E", std::fabs(x));   // d.ddddddE+XX, rounded to 7 digits
    digits[0] = buf[0];
    std::memcpy(digits + 1, buf + 2, 6);
    exp10 = std::atoi(buf + 9) + 1;                          // 0.ddddddd x 10^(XX+1)
  }
  out += neg ? "-." : "0.";
  out.append(digits, 7);
  char e[8];
  const int a = exp10 < 0 ? -exp10 : exp10;
  if (a <= 99) std::snprintf(e, sizeof e, "E%c%02d", exp10 < 0 ? '-' : '+', a);
  else if (a <= 999) std::snprintf(e, sizeof e, "%c%03d", exp10 < 0 ? '-' : '+', a);
  else std::snprintf(e, sizeof e, "****");
  out += e;
}

// Fortran Iw: right-justified in w columns, asterisks when it does not fit.
void put_i(std::string& out, long long v, int w) {
  char buf[32];
  const int n = std::snprintf(buf, sizeof buf, "%*lld", w, v);
  if (n > w) out.append((size_t)w, '*');
  else out += buf;
}

}  // namespace

SWE_API int swe_write_vtk_2d(const char* path, const char* title, int np, int me, const int* jj, const double* rr,
                             const double* field) {
  if (!path || !title || np <= 0 || me < 0 || (me > 0 && !jj) || !rr || !field) return SWE_ERR_ARG;
  std::string s;
  s.reserve((size_t)np * 52 + (size_t)me * 40 + 256);
  s += "# vtk DataFile Version 3.0\n";
  s += "vtk ";
  s += title;
  s += "\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS ";
  put_i(s, np, 7);
  s += " float\n";
  for (int i = 0; i < np; i++) {                     // '(2(e13.7,2x),A)', x, y, ' 0.0 '
    put_e13_7(s, rr[2 * (size_t)i]);
    s += "  ";
    put_e13_7(s, rr[2 * (size_t)i + 1]);
    s += "   0.0 \n";
  }
  s += "CELLS ";                                     // '(A,I7,I8)'
  put_i(s, me, 7);
  put_i(s, 4LL * me, 8);
  s += '\n';
  for (int k = 0; k < me; k++) {                     // '(A,3(I8,1x))', '3 ', jj - 1
    s += "3 ";
    for (int v = 0; v < 3; v++) {
      if (v) s += ' ';
      put_i(s, (long long)jj[3 * (size_t)k + v] - 1, 8);
    }
    s += '\n';
  }
  s += "CELL_TYPES ";
  put_i(s, me, 7);
  s += '\n';
  for (int k = 0; k < me; k++) s += "5\n";
  s += "POINT_DATA ";
  put_i(s, np, 7);
  s += "\nSCALARS scalars float 1\nLOOKUP_TABLE default\n";
  for (int i = 0; i < np; i++) {                     // '(e13.7,2x)'
    put_e13_7(s, field[i]);
    s += '\n';
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return SWE_ERR_ARG;
  const size_t wrote = std::fwrite(s.data(), 1, s.size(), f);
  const int closed = std::fclose(f);
  return (wrote == s.size() && closed == 0) ? SWE_OK : SWE_ERR_ARG;
}

// ---- gauge location (post_interp.f90: pd_scal :133-141, pd_vect :144-153,
// inside :492-524, FE_interpolation :206-255), FP64 without contraction ----
namespace {
struct V2 {
  double x, y;
};
inline V2 node(const swe::HostMesh& m, int e, int v) {
  const int n = m.jj[3 * (size_t)e + v];
  return V2{m.rr[2 * (size_t)n], m.rr[2 * (size_t)n + 1]};
}
inline V2 sub(V2 a, V2 b) { return V2{a.x - b.x, a.y - b.y}; }
inline V2 pd_vect(V2 y) { return V2{-y.y, y.x}; }
inline double pd_scal(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
}  // namespace

namespace swe {

int gauge_element(const HostMesh& m, const double* rp) {
  const V2 r{rp[0], rp[1]};
  for (int e = 0; e < m.me; e++) {
    const V2 r1 = node(m, e, 0), r2 = node(m, e, 1), r3 = node(m, e, 2);
    const double s1 = pd_scal(pd_vect(sub(r3, r2)), sub(r, r2));
    const double s2 = pd_scal(pd_vect(sub(r1, r3)), sub(r, r3));
    const double s3 = pd_scal(pd_vect(sub(r2, r1)), sub(r, r1));
    if (!(std::fmin(std::fmin(s1, s2), s3) < -1.e-12)) return e;
  }
  return -1;
}

void gauge_weights(const HostMesh& m, int e, const double* rp, double* ff) {
  const V2 r{rp[0], rp[1]};
  const V2 r1 = node(m, e, 0), r2 = node(m, e, 1), r3 = node(m, e, 2);
  const V2 n2 = pd_vect(sub(r1, r3)), n3 = pd_vect(sub(r2, r1));
  const double x = 1.0 - pd_scal(n2, sub(r2, r)) / pd_scal(n2, sub(r2, r3));
  const double y = 1.0 - pd_scal(n3, sub(r3, r)) / pd_scal(n3, sub(r3, r1));
  ff[0] = (1.0 - x) - y;
  ff[1] = x;
  ff[2] = y;
}

}  // namespace swe
