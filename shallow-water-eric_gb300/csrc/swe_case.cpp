// The reference's set-up around the step, on the host in C++ (declared in
// include/swe_case.hpp): the data-file reader, the .FEM mesh reader with the
// reference's renumbering, the Dirichlet node lists and the test cases'
// init / sol_anal.  Each function cites the reference routine it restates.
#include "../../include/swe_case.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>

namespace swe {

namespace {

[[noreturn]] void fail(const std::string& msg) { throw std::runtime_error(msg); }

std::string strip(const std::string& s) {
  const char* ws = " \t\r\n";
  const size_t a = s.find_first_not_of(ws);
  if (a == std::string::npos) return "";
  return s.substr(a, s.find_last_not_of(ws) - a + 1);
}

// read_until (tools.f90:3-19): REWIND, then the record after the first one
// whose first 128 characters, trimmed and left-adjusted, equal the marker
size_t read_until(const std::vector<std::string>& lines, const std::string& marker) {
  for (size_t i = 0; i < lines.size(); i++)
    if (strip(lines[i].substr(0, 128)) == marker) return i + 1;
  fail("Data string " + marker + " not found");
}

// one record's values, list-directed: quoted strings keep blanks (a doubled
// quote is one quote), other values end at a blank, comma or slash, r*c
// repeats c r times, a slash ends the record
std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> out;
  size_t p = 0;
  const size_t n = line.size();
  auto blank = [](char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n'; };
  while (p < n) {
    while (p < n && blank(line[p])) p++;
    if (p >= n || line[p] == '/') break;
    if (line[p] == ',') { p++; continue; }
    if (line[p] == '\'' || line[p] == '"') {
      const char q = line[p++];
      std::string v;
      while (p < n) {
        if (line[p] == q) {
          if (p + 1 < n && line[p + 1] == q) { v += q; p += 2; continue; }
          p++;
          break;
        }
        v += line[p++];
      }
      out.push_back(v);
    } else {
      const size_t a = p;
      while (p < n && !blank(line[p]) && line[p] != ',' && line[p] != '/') p++;
      const std::string tok = line.substr(a, p - a);
      const size_t star = tok.find('*');
      bool rep = star != std::string::npos && star > 0;
      for (size_t k = 0; rep && k < star; k++) rep = tok[k] >= '0' && tok[k] <= '9';
      if (rep) {
        const int r = std::stoi(tok.substr(0, star));
        for (int k = 0; k < r; k++) out.push_back(tok.substr(star + 1));
      } else {
        out.push_back(tok);
      }
    }
    while (p < n && blank(line[p])) p++;
    if (p < n && line[p] == ',') p++;
  }
  return out;
}

// n values from record i on (a list may continue on the next records)
std::vector<std::string> values(const std::vector<std::string>& lines, size_t i, size_t n) {
  std::vector<std::string> v;
  while (v.size() < n) {
    if (i >= lines.size()) fail("end of file while reading values");
    const std::vector<std::string> t = tokens(lines[i++]);
    v.insert(v.end(), t.begin(), t.end());
  }
  v.resize(n);
  return v;
}

double real_of(std::string t) {
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  size_t used = 0;
  const double v = std::stod(t, &used);
  if (used != t.size()) fail("not a real: " + t);
  return v;
}

int int_of(const std::string& t) {
  size_t used = 0;
  const int v = std::stoi(t, &used);
  if (used != t.size()) fail("not an integer: " + t);
  return v;
}

bool logical_of(const std::string& t) {
  size_t a = 0;
  while (a < t.size() && t[a] == '.') a++;
  if (a < t.size() && (t[a] == 'T' || t[a] == 't')) return true;
  if (a < t.size() && (t[a] == 'F' || t[a] == 'f')) return false;
  fail("not a logical: " + t);
}

}  // namespace

// read_my_data (read_data.f90:35-100), in its order
DataFile read_my_data(const std::string& path) {
  std::ifstream f(path);
  if (!f) fail("cannot open " + path);
  std::vector<std::string> lines;
  for (std::string l; std::getline(f, l);) lines.push_back(l);
  auto one = [&](const std::string& m) { return values(lines, read_until(lines, m), 1)[0]; };
  auto many = [&](const std::string& m, int n) {
    return n > 0 ? values(lines, read_until(lines, m), (size_t)n) : std::vector<std::string>();
  };
  auto ints = [](const std::vector<std::string>& v) {
    std::vector<int> o;
    for (const std::string& s : v) o.push_back(int_of(s));
    return o;
  };
  DataFile d;
  d.directory = one("===Name of directory for mesh file===");
  d.file_name = one("===Name of mesh file===");
  d.nb_dom = int_of(one("===Number of subdomains in the mesh==="));
  d.list_dom = ints(many("===List of subdomain in the mesh===", d.nb_dom));
  d.type_fe = int_of(one("===Type of finite element==="));
  d.Tfinal = real_of(one("===Final time==="));
  d.CFL = real_of(one("===CFL number==="));
  d.viscosity_type = one("===Viscosity type (galerkin, viscous, entropy_visc, fct)===").substr(0, 15);
  d.viscous_type = one("===Type of first-order viscosity===");
  d.if_alpha_limit = logical_of(one("===Alpha limitation? (True/False)==="));
  d.if_lumped = logical_of(one("===Lumping the mass matrix? (true/false)==="));
  d.type_test = int_of(one("===Test case number==="));
  const char* comp[3] = {"h", "ux", "uy"};
  std::vector<int>* lists[3] = {&d.h_Dir_list, &d.ux_Dir_list, &d.uy_Dir_list};
  for (int c = 0; c < 3; c++) {
    const int n = int_of(one(std::string("===How many Dirichlet boundaries for ") + comp[c] + "?==="));
    *lists[c] = ints(many(std::string("===List of Dirichlet boundaries for ") + comp[c] + "?===", n));
  }
  if (d.type_test == 9 || d.type_test == 10) d.mannings = real_of(one("===Mannings coefficient==="));
  if (d.type_test == 13) d.lambdaSGN = real_of(one("===Lambda for SGN model==="));
  return d;
}

// load_mesh_free_format (prep_mesh.f90:759-1035) for P1 triangles: the
// gfortran sequential records (4-byte length markers) of np, nw, me, nws,
// mes / jj, neigh, i_d / jjs, neighs, sides / rr; elements of the listed
// domains are kept in file order and their nodes renumbered by first touch;
// a boundary side is kept when its element, or the element across it, is in
// a listed domain
FemMesh load_mesh_free_format(const std::string& path, const std::vector<int>& list_dom) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail("cannot open " + path);
  std::vector<char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::vector<std::pair<size_t, size_t>> rec;   // (offset, length)
  size_t off = 0;
  while (off < buf.size()) {
    int32_t n1 = 0, n2 = 0;
    if (off + 4 > buf.size()) fail("corrupt record markers in .FEM file");
    std::memcpy(&n1, &buf[off], 4);
    if (n1 < 0 || off + 8 + (size_t)n1 > buf.size()) fail("corrupt record markers in .FEM file");
    std::memcpy(&n2, &buf[off + 4 + n1], 4);
    if (n2 != n1) fail("corrupt record markers in .FEM file");
    rec.emplace_back(off + 4, (size_t)n1);
    off += 8 + (size_t)n1;
  }
  if (rec.size() < 4 || rec[0].second < 20) fail("a .FEM file has four records");
  int32_t hd[5];
  std::memcpy(hd, &buf[rec[0].first], 20);
  const int np0 = hd[0], nw = hd[1], me0 = hd[2], nws = hd[3], mes0 = hd[4];
  if (nw != 3 || nws != 2) fail("only P1 triangle meshes are supported");
  if (np0 <= 0 || me0 <= 0 || mes0 < 0) fail("bad sizes in .FEM file header");
  auto ints = [&](int r, size_t count) {
    if (rec[r].second < count * 4) fail("short record in .FEM file");
    std::vector<int32_t> v(count);
    std::memcpy(v.data(), &buf[rec[r].first], count * 4);
    return v;
  };
  const std::vector<int32_t> a = ints(1, 7 * (size_t)me0);
  const std::vector<int32_t> b = ints(2, 4 * (size_t)mes0);
  if (rec[3].second < 16 * (size_t)np0) fail("short record in .FEM file");
  std::vector<double> rr0(2 * (size_t)np0);
  std::memcpy(rr0.data(), &buf[rec[3].first], rr0.size() * 8);
  const int32_t* jj0 = a.data();                  // (3, me)
  const int32_t* neigh0 = a.data() + 3 * (size_t)me0;
  const int32_t* id0 = a.data() + 6 * (size_t)me0;
  const int32_t* jjs0 = b.data();                 // (2, mes)
  const int32_t* neighs0 = b.data() + 2 * (size_t)mes0;
  const int32_t* sides0 = b.data() + 3 * (size_t)mes0;
  auto in_dom = [&](int m) {                      // m 1-based
    return std::find(list_dom.begin(), list_dom.end(), id0[m - 1]) != list_dom.end();
  };
  std::vector<int> nouv_nd(np0 + 1, 0), ancien_nd;
  FemMesh m;
  for (int e = 0; e < me0; e++) {
    if (!in_dom(e + 1)) continue;
    for (int n = 0; n < 3; n++) {
      const int i = jj0[3 * (size_t)e + n];
      if (i < 1 || i > np0) fail("node number out of range in .FEM file");
      if (nouv_nd[i] == 0) {
        ancien_nd.push_back(i);
        nouv_nd[i] = (int)ancien_nd.size();
      }
      m.jj.push_back(nouv_nd[i]);
    }
  }
  m.me = (int)m.jj.size() / 3;
  m.np = (int)ancien_nd.size();
  for (int s = 0; s < mes0; s++) {
    const int m1 = neighs0[s];
    if (m1 < 1 || m1 > me0) fail("side element out of range in .FEM file");
    bool ok = in_dom(m1);
    if (!ok) {
      int n = 0;
      for (; n < 3; n++) {
        const int v = jj0[3 * (size_t)(m1 - 1) + n];
        if (v != jjs0[2 * (size_t)s] && v != jjs0[2 * (size_t)s + 1]) break;
      }
      const int m2 = neigh0[3 * (size_t)(m1 - 1) + (n < 3 ? n : 2)];
      if (m2 < 0 || m2 > me0) fail("neighbour element out of range in .FEM file");
      ok = m2 != 0 && in_dom(m2);
    }
    if (!ok) continue;
    for (int q = 0; q < 2; q++) {
      const int v = jjs0[2 * (size_t)s + q];
      if (v < 1 || v > np0) fail("side node out of range in .FEM file");
      m.jjs.push_back(nouv_nd[v]);
    }
    m.sides.push_back(sides0[s]);
  }
  m.mes = (int)m.sides.size();
  m.rr.resize(2 * (size_t)m.np);
  for (int i = 0; i < m.np; i++) {
    m.rr[2 * (size_t)i] = rr0[2 * (size_t)(ancien_nd[i] - 1)];
    m.rr[2 * (size_t)i + 1] = rr0[2 * (size_t)(ancien_nd[i] - 1) + 1];
  }
  return m;
}

// dirichlet_nodes (dir_nodes.f90:243-292,495-511): the sorted unique nodes of
// the boundary edges whose side is listed
std::vector<int> dirichlet_nodes(const FemMesh& m, const std::vector<int>& sides) {
  std::vector<int> js;
  for (int s = 0; s < m.mes; s++)
    if (std::find(sides.begin(), sides.end(), m.sides[s]) != sides.end()) {
      js.push_back(m.jjs[2 * (size_t)s]);
      js.push_back(m.jjs[2 * (size_t)s + 1]);
    }
  std::sort(js.begin(), js.end());
  js.erase(std::unique(js.begin(), js.end()), js.end());
  return js;
}

// ---------------------------------------------------------------------------
// init / sol_anal (condlim.f90).  Integer powers are products and real
// powers pow(), as Fortran evaluates them; default-real literals (h0 = 0.32
// of type 8) are single precision.
// ---------------------------------------------------------------------------
namespace {

const double kH0Island = (double)0.32f;

double bump(double x) {   // 0.2*(x-8)**3*(12-x)**3/64
  const double a = x - 8.0, b = 12.0 - x;
  return 0.2 * ((a * a) * a) * ((b * b) * b) / 64.0;
}

double paraboloid(double x, double y, double h0, double hL, double a) {
  const double dx = x - hL / 2.0, dy = y - hL / 2.0;
  return -h0 * (1.0 - (dx * dx + dy * dy) / (a * a));
}

struct Cubic {
  double R, Q, D;
};

Cubic cardano(double b, double d) {   // x**3 + b x**2 + d = 0 as sol_anal writes it
  Cubic c;
  c.R = (-27 * d - 2 * ((b * b) * b)) / 54;
  c.Q = -(b * b) / 9;
  c.D = (c.Q * c.Q) * c.Q + c.R * c.R;
  return c;
}

void trig_roots(const Cubic& c, double b, double* x1, double* x2, double* x3) {
  const double tpio3 = 2 * std::acos(-1.0) / 3, fpio3 = 2 * tpio3;
  const double theta = std::acos(c.R / std::sqrt(-((c.Q * c.Q) * c.Q)));
  const double sq = 2 * std::sqrt(-c.Q);
  *x1 = sq * std::cos(theta / 3) - b / 3;
  *x2 = sq * std::cos(theta / 3 + tpio3) - b / 3;
  *x3 = sq * std::cos(theta / 3 + fpio3) - b / 3;
}

double cardano_x2(const Cubic& c, double b) {
  const double S = -std::pow(-std::sqrt(c.D) - c.R, 1.0 / 3);
  const double T = -std::pow(std::sqrt(c.D) - c.R, 1.0 / 3);
  return -(S + T) / 2.0 - b / 3.0;
}

}  // namespace

CaseInit init_case(int tt, const FemMesh& m, double epsilon) {
  CaseInit ci;
  ci.bath.assign(m.np, 0.0);
  const double* rr = m.rr.data();
  switch (tt) {
    case 1: {                                             // condlim.f90:116-133
      ci.gravity = 1.0;
      ci.max_water_h = 0.2;
      const double e1 = std::exp(-1.0), e2 = std::exp(-2.0);
      for (int i = 0; i < m.np; i++) {
        const double x = rr[2 * (size_t)i], y = rr[2 * (size_t)i + 1];
        const double dx1 = x - 1.2, dy1 = y - 0.7, dx2 = x - 0.45, dy2 = y - 0.4;
        const double ray1 = 25.0 * (dx1 * dx1) + 50.0 * (dy1 * dy1);
        const double ray2 = 50.0 * (dx2 * dx2) + 100.0 * (dy2 * dy2);
        if (ray1 <= 2.0) {
          ci.bath[i] = ((std::exp(-ray1) - e1) / (e2 - e1) - 1.0) * (-0.2);
          if (std::fabs(std::sqrt(ray1) - 1.0) < 1.e-10) ci.bath[i] = 0.2;
        } else if (ray2 <= 1.0) {
          ci.bath[i] = -0.5 * (std::exp(-ray2) - e1);
        }
      }
      break;
    }
    case 2: case 3: case 6: case 7:                       // :134-146
      ci.max_water_h = tt == 2 ? 0.2 : 2.0;
      for (int i = 0; i < m.np; i++) {
        const double x = rr[2 * (size_t)i];
        ci.bath[i] = (8.0 < x && x < 12.0) ? bump(x) : 0.0;
      }
      break;
    case 4:                                               // :147-152
      ci.t0 = 1.0;
      ci.max_water_h = 0.005;
      break;
    case 5: {                                             // :153-163
      const double a = 1.0, h0 = 0.1, hL = 4.0;
      ci.max_water_h = hL;
      const double omega = std::sqrt(2 * ci.gravity * h0) / a;
      ci.tfinal = 6.0 * std::acos(-1.0) / omega;
      ci.sets_tfinal = true;
      for (int i = 0; i < m.np; i++) ci.bath[i] = paraboloid(rr[2 * (size_t)i], rr[2 * (size_t)i + 1], h0, hL, a);
      break;
    }
    case 8: {                                             // :164-179
      const double htop = 0.625, rcone = 3.6, scone = 4.0, hcone = 0.9;
      ci.max_water_h = kH0Island;
      for (int i = 0; i < m.np; i++) {
        const double dx = rr[2 * (size_t)i] - 15.0, dy = rr[2 * (size_t)i + 1] - 13.0;
        const double radius = std::sqrt(dx * dx + dy * dy);
        ci.bath[i] = radius < rcone ? std::min(htop, hcone - radius / scone) : 0.0;
      }
      break;
    }
    case 11: {                                            // :200-211
      const double a = 1.0, h0 = 0.1, hL = 4.0, kappa = 0.2;
      ci.max_water_h = hL;
      const double p = std::sqrt((8 * ci.gravity * h0) / (a * a));
      const double s = 1.0 / 2.0 * std::sqrt(p * p - kappa * kappa);
      ci.tfinal = 2 * 2 * std::acos(-1.0) / s;
      ci.sets_tfinal = true;
      for (int i = 0; i < m.np; i++) ci.bath[i] = paraboloid(rr[2 * (size_t)i], rr[2 * (size_t)i + 1], h0, hL, a);
      break;
    }
    case 12:                                              // :212-218
      ci.max_water_h = 6.0;
      for (int i = 0; i < m.np; i++) ci.bath[i] = paraboloid(rr[2 * (size_t)i], rr[2 * (size_t)i + 1], 0.5, 0.0, 3.0);
      break;
    case 13:                                              // :219-229
      ci.max_water_h = 11.0 / 100.0;
      break;
    case 9:
      fail("type_test 9 (Malpasset) needs malpasset.wh/.jj/.bath, which the reference does not ship");
    default:
      fail("type_test " + std::to_string(tt) + ": no init for this case (the reference STOPs: BUG in init)");
  }
  ci.htiny = epsilon * ci.max_water_h;
  return ci;
}

void sol_anal(int tt, int k, int n, const double* rr, double t, const double* bath, double g, double htiny,
              double* out) {
  auto X = [&](int i) { return rr[2 * (size_t)i]; };
  auto Y = [&](int i) { return rr[2 * (size_t)i + 1]; };
  auto zero = [&]() { std::fill(out, out + n, 0.0); };
  switch (tt) {
    case 1: case 2: {                                     // :327-345
      if (k != 1) return zero();
      const double lvl = tt == 1 ? 0.2 : 0.1;
      for (int i = 0; i < n; i++) out[i] = std::max(std::max(bath[i], lvl) - bath[i], 0.0);
      return;
    }
    case 3: {                                             // :346-379
      const double q0 = 4.42, hL = 2.0;
      if (k == 1) {
        for (int i = 0; i < n; i++) {
          const double bathi = std::max(0.0, bump(X(i)));
          if (t <= 1.e-14) { out[i] = hL - bathi; continue; }
          const double b = bathi - (q0 * q0) / (2 * g * (hL * hL)) - hL;
          const double d = (q0 * q0) / (2 * g);
          double x1, x2, x3;
          trig_roots(cardano(b, d), b, &x1, &x2, &x3);
          out[i] = x1;
        }
        return;
      }
      if (k == 2) { std::fill(out, out + n, t <= 1.e-14 ? 0.0 : q0); return; }
      return zero();
    }
    case 4: {                                             // :380-420
      const double x0 = 5.0, hL = 0.005, speed = std::sqrt(g * hL);
      if (k == 1) {
        for (int i = 0; i < n; i++) {
          if (t <= 1.e-14) { out[i] = X(i) <= x0 ? hL : 0.0; continue; }
          const double x = X(i) - x0, s = speed - x / (2 * t);
          out[i] = x <= -t * speed ? hL : (x <= 2 * t * speed ? (4.0 / (9.0 * g)) * (s * s) : 0.0 + htiny);
        }
        return;
      }
      if (k == 2) {
        for (int i = 0; i < n; i++) {
          if (t <= 1.e-14) { out[i] = 0.0; continue; }
          const double x = X(i) - x0, s = speed - x / (2 * t);
          out[i] = x <= -t * speed ? 0.0 : (x <= 2 * t * speed ? (8.0 / (27.0 * g)) * (speed + x / t) * (s * s) : 0.0);
        }
        return;
      }
      return zero();
    }
    case 5: {                                             // :421-456 (with the current +htiny film)
      const double a = 1.0, h0 = 0.1, hL = 4.0, eta = 0.5;
      const double omega = std::sqrt(2 * g * h0) / a;
      const double cs = std::cos(omega * t), sn = std::sin(omega * t);
      for (int i = 0; i < n; i++) {
        const double dx = X(i) - hL / 2.0, dy = Y(i) - hL / 2.0;
        const double bathi = -h0 * (1.0 - (dx * dx + dy * dy) / (a * a));
        const double base = std::max((eta * h0 / (a * a)) * (2.0 * dx * cs + 2.0 * dy * sn) - bathi, 0.0);
        out[i] = k == 1 ? base + htiny : k == 2 ? -eta * omega * sn * base : k == 3 ? eta * omega * cs * base : 0.0;
      }
      return;
    }
    case 6: case 7: {                                     // :457-603
      const double q0 = tt == 6 ? 1.53 : 0.18;
      const double d = (q0 * q0) / (2 * g);
      const double eta = -std::pow(27 * d / 4, 1.0 / 3);
      const double ber = 0.2 - eta;
      if (k == 2) {
        std::fill(out, out + n, (tt == 6 && t <= 1.e-14) ? 0.0 : q0);
        return;
      }
      if (k != 1) return zero();
      if (tt == 6) {
        const double x0 = 10.0, hL = 0.66;
        for (int i = 0; i < n; i++) {
          const double bathi = std::max(0.0, bump(X(i)));
          if (t <= 1.e-14) { out[i] = hL - bathi; continue; }
          const double b = bathi - ber;
          const Cubic c = cardano(b, d);
          if (c.D >= 0.0) { out[i] = cardano_x2(c, b); continue; }
          double x1, x2, x3;
          trig_roots(c, b, &x1, &x2, &x3);
          out[i] = X(i) < x0 ? std::max(x1, x3) : std::min(x1, x3);
        }
        return;
      }
      const double x0 = 10.0, xshock = 11.7;
      const double bath_shock = (8.0 < xshock && xshock < 12.0) ? bump(xshock) : 0.0;
      const double bs = bath_shock - ber;
      const Cubic cs = cardano(bs, d);
      if (cs.D >= 0.0) fail("sol_anal type 7: no pre-shock root (the reference prints BUG case(7))");
      double s1, s2, s3;
      trig_roots(cs, bs, &s1, &s2, &s3);
      const double h_post = (-s3 + std::sqrt(s3 * s3 + 8 * (q0 * q0) / (g * s3))) / 2;
      for (int i = 0; i < n; i++) {
        const double bathi = std::max(0.0, bump(X(i)));
        if (t <= 1.e-14) { out[i] = h_post - bathi; continue; }
        const double b = bathi - ber;
        const Cubic c = cardano(b, d);
        if (c.D >= 0.0) { out[i] = cardano_x2(c, b); continue; }
        double x1, x2, x3;
        trig_roots(c, b, &x1, &x2, &x3);
        out[i] = X(i) < x0 ? std::max(x1, x3) : X(i) < xshock ? std::min(x1, x3) : bath_shock + h_post - bathi;
      }
      return;
    }
    case 8: {                                             // :604-628
      const double h0 = kH0Island, alpha = 1 * h0, xs = 15.0 - 12.96;
      const double vel = std::sqrt(3.0 * alpha / (4 * ((h0 * h0) * h0)));
      for (int i = 0; i < n; i++) {
        const double ch = std::cosh(vel * (X(i) - xs));
        if (k == 1) out[i] = t <= 1.e-14 ? std::max(h0 + alpha / (ch * ch) - bath[i], 0.0) : h0;
        else if (k == 2) out[i] = t <= 1.e-14 ? alpha / (ch * ch) * std::sqrt(g / h0) : 0.0;
        else out[i] = 0.0;
      }
      return;
    }
    case 11: {                                            // :645-697
      if (k > 3) fail("sol_anal type 11 has no component " + std::to_string(k));
      const double a = 1.0, h0 = 0.1, hL = 4.0, kappa = 0.2, gamma = 0.5;
      const double p = std::sqrt((8 * g * h0) / (a * a));
      const double s = 1.0 / 2.0 * std::sqrt(p * p - kappa * kappa);
      const double e2 = std::exp(-kappa * t / 2.0), cs = std::cos(s * t), sn = std::sin(s * t);
      for (int i = 0; i < n; i++) {
        const double bathi = paraboloid(X(i), Y(i), h0, hL, a);
        const double htilde = -bathi - (gamma * gamma) / (2 * g) * std::exp(-kappa * t) -
                              gamma / (2.0 * g) * e2 * (X(i) - hL / 2.0) * (2 * s * cs + kappa * sn) -
                              gamma / (2.0 * g) * e2 * (Y(i) - hL / 2.0) * (kappa * cs - 2.0 * s * sn);
        const double h = std::max(htilde, 0.0);
        out[i] = k == 1 ? h : k == 2 ? h * gamma * e2 * sn : h * gamma * e2 * cs;
      }
      return;
    }
    case 12: {                                            // :698-750
      if (k > 3) fail("sol_anal type 12 has no component " + std::to_string(k));
      const double a = 3.0, h0 = 0.5, hL = 0.0, f = 2.0, eta = 0.5;
      const double a2 = a * a, a4 = a2 * a2;
      const double den = (f * f) * a4 + std::sqrt(8.0 * (f * f) * g * h0 * (a4 * a2) + ((f * f) * (f * f)) * (a4 * a4));
      const double delta = 2.0 * f * a4 / den;
      const double w = -1.0 / (std::sqrt(2.0) * a2) * std::sqrt(4.0 * g * h0 * a2 + den);
      const double cs = std::cos(w * t), sn = std::sin(w * t);
      for (int i = 0; i < n; i++) {
        const double bathi = paraboloid(X(i), Y(i), h0, hL, a);
        const double htilde = -bathi - eta / g * cs * (1 - delta * f) * (Y(i) - hL / 2.0) +
                              eta / g * sn * (f / w - delta * w) * (X(i) - hL / 2.0) +
                              (eta * eta) / (2.0 * g) * ((delta * delta) * cs * cs + sn * sn / (w * w));
        const double h = std::max(htilde, 0.0);
        out[i] = k == 1 ? h : k == 2 ? -h * delta * eta * cs : h * eta * sn / w;
      }
      return;
    }
    case 13: {                                            // :751-824
      if ((k == 4 || k == 5) && t > 1.e-10)
        fail("sol_anal type 13 leaves component " + std::to_string(k) + " undefined for t > 1e-10");
      const double h1 = 10.0 / 100.0, h2 = 11.0 / 100.0, x0 = 2.75;
      const double D = std::sqrt(g * h2);
      const double z = std::sqrt((3.0 * (h2 - h1)) / (h2 * std::pow(h1, 2.0)));
      for (int i = 0; i < n; i++) {
        const double arg = 1.0 / 2.0 * z * (X(i) - x0 - D * t);
        const double se = 1.0 / std::cosh(arg), se2 = se * se;
        const double ht = std::max(h1 + (h2 - h1) * se2, 0.0);
        out[i] = k == 1 ? ht : k == 2 ? ht * D - h1 * D : k == 3 ? ht * 0.0 : k == 4 ? ht * ht
               : -D * h1 * ((h1 - h2) * z * se2 * std::tanh(arg));
      }
      return;
    }
    default:
      fail("type_test " + std::to_string(tt) + ": no sol_anal for this case (the reference STOPs)");
  }
}

}  // namespace swe
