// Device-side setup: the CSR pattern of st_csr and the mass / c_ij / lumped
// assembly of construct_matrices on the GPU.
//
// One thread owns one node's CSR row.  Its incident elements are visited in
// ascending element order and each contribution is added with the same
// expression as the reference's element loops (SOURCES/update.f90:18-132,
// SFEMaNS/FEMSUB_OBJET/fem_sparsekit.f90:6-53, gauss_points_2d_p1.f90:95-128,
// 347-393), so every entry receives the same sequence of FP64 additions as in
// the reference and the matrices are bit-identical (this unit is compiled
// with -fmad=false).  The two prefix sums (element offsets, row offsets) run
// on the host: they are a few MB.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "swe_setup.hpp"

namespace swe {
namespace {

// st_csr caps a row at nparm = 90 entries and nothing else; a node can then
// lie in at most C(89, 2) distinct triangles, so a node listed in more
// elements than that repeats an element.  The guard bounds the per-node sort.
constexpr int kMaxElemsPerNode = 4096;
constexpr int kNparm = 90;             // st_csr's row cap (st_sparsekit.f90:801)

enum : int { SE_RANGE = 1, SE_ELEMS = 2, SE_ROW = 4, SE_LUMPED = 8 };

__global__ void k_count_elems(const int* __restrict__ jj, int me, int np, int* __restrict__ cnt,
                              int* __restrict__ err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= me) return;
  for (int n = 0; n < 3; n++) {
    const int v = jj[3 * e + n];
    if (v < 0 || v >= np) { atomicOr(err, SE_RANGE); continue; }
    atomicAdd(&cnt[v], 1);
  }
}

__global__ void k_fill_elems(const int* __restrict__ jj, int me, int np, const int* __restrict__ eoff,
                             int* __restrict__ fillc, int* __restrict__ elist) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= me) return;
  for (int n = 0; n < 3; n++) {
    const int v = jj[3 * e + n];
    if (v < 0 || v >= np) continue;
    elist[eoff[v] + atomicAdd(&fillc[v], 1)] = e;
  }
}

// Node i's row of st_csr: i and every node of its elements, ascending,
// without repeats (st_sparsekit.f90:788-863).  Sorts the node's element list
// in place (ascending element index) on the way.  Returns the row length, or
// -1 past the caps.
__device__ int row_of(const int* __restrict__ jj, int* __restrict__ elist, int b, int k, int i, int* buf) {
  if (k > kMaxElemsPerNode) return -1;
  for (int a = 1; a < k; a++) {              // insertion sort of the element list
    const int x = elist[b + a];
    int c = a - 1;
    while (c >= 0 && elist[b + c] > x) { elist[b + c + 1] = elist[b + c]; c--; }
    elist[b + c + 1] = x;
  }
  int n = 0;
  buf[n++] = i;
  for (int a = 0; a < k; a++)
    for (int q = 0; q < 3; q++) {
      const int v = jj[3 * elist[b + a] + q];
      int c = n - 1;                         // insert v keeping buf sorted and unique
      bool dup = false;
      while (c >= 0 && buf[c] >= v) { if (buf[c] == v) { dup = true; break; } c--; }
      if (dup) continue;
      if (n >= kNparm) return -1;
      for (int t = n; t > c + 1; t--) buf[t] = buf[t - 1];
      buf[c + 1] = v;
      n++;
    }
  return n;
}

__global__ void k_row_len(const int* __restrict__ jj, int np, const int* __restrict__ eoff, int* __restrict__ elist,
                          int* __restrict__ rowlen, int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int buf[kNparm];
  const int b = eoff[i], k = eoff[i + 1] - b;
  const int n = row_of(jj, elist, b, k, i, buf);
  if (n < 0) atomicOr(err, k > kMaxElemsPerNode ? SE_ELEMS : SE_ROW);
  rowlen[i] = n < 0 ? 0 : n;
}

__global__ void k_row_fill(const int* __restrict__ jj, int np, const int* __restrict__ eoff, int* __restrict__ elist,
                           const int* __restrict__ ia, int* __restrict__ ja) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int buf[kNparm];
  const int b = eoff[i], k = eoff[i + 1] - b;
  const int n = row_of(jj, elist, b, k, i, buf);
  for (int q = 0; q < n; q++) ja[ia[i] + q] = buf[q];
}

__device__ __forceinline__ int find_in_row(const int* __restrict__ ja, int p0, int p1, int j) {
  for (int p = p0; p < p1; p++) if (ja[p] == j) return p;
  return -1;
}

// Mass, c_ij, lumped and diag of row i.  The reference adds, per element in
// ascending order, mass[p] += ww[nj][l] (1 rj[l]) ww[ni][l] for l = 1..3 and
// c_ij[p] += sum_l dw[l][nj] ww[ni][l] rj[l]; row i only sees ni = its own
// local index, in the same element order.
__global__ void k_assemble(const int* __restrict__ jj, const double* __restrict__ rr, int np,
                           const int* __restrict__ eoff, const int* __restrict__ elist, const int* __restrict__ ia,
                           const int* __restrict__ ja, double* __restrict__ mass, double* __restrict__ cx,
                           double* __restrict__ cy, double* __restrict__ lumped, int* __restrict__ diag,
                           int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double one = 1, two = 2, three = 3, six = 6;
  const double xx[3] = {one / six, two / three, one / six};
  const double yy[3] = {one / six, one / six, two / three};
  const double dd[2][3] = {{-one, one, 0.0}, {-one, 0.0, one}};
  double ww[3][3];
  for (int l = 0; l < 3; l++) { ww[0][l] = one - xx[l] - yy[l]; ww[1][l] = xx[l]; ww[2][l] = yy[l]; }
  const double pp = one / six;
  const int p0 = ia[i], p1 = ia[i + 1];
  for (int p = p0; p < p1; p++) { mass[p] = 0.0; cx[p] = 0.0; cy[p] = 0.0; }
  for (int a = eoff[i]; a < eoff[i + 1]; a++) {
    const int e = elist[a];
    const int nd[3] = {jj[3 * e], jj[3 * e + 1], jj[3 * e + 2]};
    const int ni = (nd[0] == i) ? 0 : (nd[1] == i) ? 1 : 2;
    double dw[3][3][2], rj[3];
    for (int l = 0; l < 3; l++) {
      double dr[2][2];
      for (int k = 0; k < 2; k++)
        for (int k1 = 0; k1 < 2; k1++) {
          double s = 0.0;
          for (int n = 0; n < 3; n++) s = s + rr[(size_t)nd[n] * 2 + k] * dd[k1][n];
          dr[k][k1] = s;
        }
      const double rjac = dr[0][0] * dr[1][1] - dr[0][1] * dr[1][0];
      for (int n = 0; n < 3; n++) {
        dw[l][n][0] = (+dd[0][n] * dr[1][1] - dd[1][n] * dr[1][0]) / rjac;
        dw[l][n][1] = (-dd[0][n] * dr[0][1] + dd[1][n] * dr[0][0]) / rjac;
      }
      rj[l] = rjac * pp;
    }
    for (int l = 0; l < 3; l++) {
      const double al = 1.0 * rj[l];
      for (int nj = 0; nj < 3; nj++) {
        const double x = ww[nj][l] * al * ww[ni][l];
        const int p = find_in_row(ja, p0, p1, nd[nj]);
        mass[p] = mass[p] + x;
      }
    }
    for (int nj = 0; nj < 3; nj++) {
      double x[2];
      for (int d = 0; d < 2; d++) {
        double s = 0.0;
        for (int l = 0; l < 3; l++) s = s + dw[l][nj][d] * ww[ni][l] * rj[l];
        x[d] = s;
      }
      const int p = find_in_row(ja, p0, p1, nd[nj]);
      cx[p] = cx[p] + x[0];
      cy[p] = cy[p] + x[1];
    }
  }
  double s = 0.0;
  for (int p = p0; p < p1; p++) s = s + mass[p];
  lumped[i] = s;
  diag[i] = find_in_row(ja, p0, p1, i);
  if (!(s > 0.0)) atomicOr(err, SE_LUMPED);
}

template <typename T>
cudaError_t dalloc(T** p, size_t n) { return cudaMalloc(reinterpret_cast<void**>(p), (n ? n : 1) * sizeof(T)); }

}  // namespace

std::string construct_matrices_device(HostMesh& m) {
  const int np = m.np, me = m.me;
  int *d_jj = nullptr, *d_cnt = nullptr, *d_eoff = nullptr, *d_elist = nullptr, *d_err = nullptr;
  int *d_rowlen = nullptr, *d_ia = nullptr, *d_ja = nullptr, *d_diag = nullptr;
  double *d_rr = nullptr, *d_mass = nullptr, *d_cx = nullptr, *d_cy = nullptr, *d_lumped = nullptr;
  std::string msg;
  cudaError_t st = cudaSuccess;
  auto ok = [&](cudaError_t e) { if (st == cudaSuccess && e != cudaSuccess) st = e; return st == cudaSuccess; };
  const unsigned be = (unsigned)((me + 127) / 128), bn = (unsigned)((np + 127) / 128);
  int herr = 0;
  std::vector<int> h(np + 1);
  if (ok(dalloc(&d_jj, 3 * (size_t)me)) && ok(dalloc(&d_rr, 2 * (size_t)np)) && ok(dalloc(&d_cnt, np)) &&
      ok(dalloc(&d_eoff, np + 1)) && ok(dalloc(&d_elist, 3 * (size_t)me)) && ok(dalloc(&d_err, 1)) &&
      ok(dalloc(&d_rowlen, np)) && ok(dalloc(&d_ia, np + 1)) && ok(dalloc(&d_lumped, np)) &&
      ok(dalloc(&d_diag, np)) &&
      ok(cudaMemcpy(d_jj, m.jj.data(), 3 * (size_t)me * sizeof(int), cudaMemcpyHostToDevice)) &&
      ok(cudaMemcpy(d_rr, m.rr.data(), 2 * (size_t)np * sizeof(double), cudaMemcpyHostToDevice)) &&
      ok(cudaMemset(d_cnt, 0, np * sizeof(int))) && ok(cudaMemset(d_err, 0, sizeof(int)))) {
    k_count_elems<<<be, 128>>>(d_jj, me, np, d_cnt, d_err);
    // element offsets: host prefix sum of the counts
    if (ok(cudaGetLastError()) && ok(cudaMemcpy(h.data(), d_cnt, np * sizeof(int), cudaMemcpyDeviceToHost))) {
      int acc = 0;
      for (int i = 0; i < np; i++) { const int c = h[i]; h[i] = acc; acc += c; }
      h[np] = acc;
      if (ok(cudaMemcpy(d_eoff, h.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice)) &&
          ok(cudaMemset(d_cnt, 0, np * sizeof(int)))) {
        k_fill_elems<<<be, 128>>>(d_jj, me, np, d_eoff, d_cnt, d_elist);
        k_row_len<<<bn, 128>>>(d_jj, np, d_eoff, d_elist, d_rowlen, d_err);
      }
    }
    // row offsets
    if (ok(cudaGetLastError()) && ok(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost)) && herr == 0 &&
        ok(cudaMemcpy(h.data(), d_rowlen, np * sizeof(int), cudaMemcpyDeviceToHost))) {
      m.ia.assign(np + 1, 0);
      for (int i = 0; i < np; i++) m.ia[i + 1] = m.ia[i] + h[i];
      const size_t nnz = (size_t)m.ia[np];
      if (ok(cudaMemcpy(d_ia, m.ia.data(), (np + 1) * sizeof(int), cudaMemcpyHostToDevice)) &&
          ok(dalloc(&d_ja, nnz)) && ok(dalloc(&d_mass, nnz)) && ok(dalloc(&d_cx, nnz)) && ok(dalloc(&d_cy, nnz))) {
        k_row_fill<<<bn, 128>>>(d_jj, np, d_eoff, d_elist, d_ia, d_ja);
        k_assemble<<<bn, 128>>>(d_jj, d_rr, np, d_eoff, d_elist, d_ia, d_ja, d_mass, d_cx, d_cy, d_lumped, d_diag,
                                d_err);
        m.ja.resize(nnz); m.mass.resize(nnz); m.cx.resize(nnz); m.cy.resize(nnz);
        m.lumped.resize(np); m.diag.resize(np);
        ok(cudaGetLastError());
        ok(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.ja.data(), d_ja, nnz * sizeof(int), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.mass.data(), d_mass, nnz * sizeof(double), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.cx.data(), d_cx, nnz * sizeof(double), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.cy.data(), d_cy, nnz * sizeof(double), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.lumped.data(), d_lumped, np * sizeof(double), cudaMemcpyDeviceToHost));
        ok(cudaMemcpy(m.diag.data(), d_diag, np * sizeof(int), cudaMemcpyDeviceToHost));
      }
    }
  }
  if (st != cudaSuccess) msg = std::string("device setup: ") + cudaGetErrorString(st);
  else if (herr & SE_RANGE) msg = "element node index out of range";
  else if (herr & SE_ELEMS) msg = "a node belongs to more than 4096 elements (repeated elements)";
  else if (herr & SE_ROW) msg = "a CSR row exceeds 90 entries (st_csr nparm)";
  else if (herr & SE_LUMPED) msg = "non-positive lumped mass (clockwise or degenerate triangle)";
  for (void* p : {(void*)d_jj, (void*)d_cnt, (void*)d_eoff, (void*)d_elist, (void*)d_err, (void*)d_rowlen,
                  (void*)d_ia, (void*)d_ja, (void*)d_diag, (void*)d_rr, (void*)d_mass, (void*)d_cx, (void*)d_cy,
                  (void*)d_lumped})
    if (p) cudaFree(p);
  return msg;
}

}  // namespace swe
