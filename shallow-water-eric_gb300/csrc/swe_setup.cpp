// Host-side setup: the renumbering (Morton or RCM, then rows sorted by length
// in small windows) and the GB300 edge-graph layout of matrices assembled on
// the device (swe_setup_gpu.cu).
#include "swe_setup.hpp"

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <numeric>
#include <queue>
#include <string>

namespace swe {

void gauss_points(const HostMesh& m, double* rj, double* rr_gauss) {
  const double one = 1, two = 2, three = 3, six = 6;
  const double xx[3] = {one / six, two / three, one / six};
  const double yy[3] = {one / six, one / six, two / three};
  const double dd[2][3] = {{-one, one, 0.0}, {-one, 0.0, one}};
  double ww[3][3];
  for (int l = 0; l < 3; l++) { ww[0][l] = one - xx[l] - yy[l]; ww[1][l] = xx[l]; ww[2][l] = yy[l]; }
  const double pp = one / six;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < m.me; e++) {
    const int nd[3] = {m.jj[e * 3], m.jj[e * 3 + 1], m.jj[e * 3 + 2]};
    for (int l = 0; l < 3; l++) {
      double dr[2][2];
      for (int k = 0; k < 2; k++)
        for (int k1 = 0; k1 < 2; k1++) {
          double s = 0.0;
          for (int n = 0; n < 3; n++) s = s + m.rr[(size_t)nd[n] * 2 + k] * dd[k1][n];
          dr[k][k1] = s;
        }
      const double rjac = dr[0][0] * dr[1][1] - dr[0][1] * dr[1][0];
      if (rj) rj[(size_t)e * 3 + l] = rjac * pp;
      if (rr_gauss)
        for (int k = 0; k < 2; k++) {
          double s = 0.0;
          for (int n = 0; n < 3; n++) s = s + ww[n][l] * m.rr[(size_t)nd[n] * 2 + k];
          rr_gauss[((size_t)e * 3 + l) * 2 + k] = s;
        }
    }
  }
}

// Reverse Cuthill-McKee: BFS from a pseudo-peripheral node of each connected
// component, neighbours visited by increasing degree, order reversed.
std::vector<int> rcm_order(const HostMesh& m) {
  const int n = m.np;
  std::vector<int> deg(n);
  for (int i = 0; i < n; i++) deg[i] = m.ia[i + 1] - m.ia[i] - 1;
  std::vector<int> order;
  order.reserve(n);
  std::vector<char> seen(n, 0);
  std::vector<int> level(n, -1);
  auto bfs_far = [&](int s) {   // farthest node of minimal degree from s
    std::vector<int> q{s};
    std::vector<int> touched{s};
    level[s] = 0;
    size_t h = 0;
    int far = s;
    while (h < q.size()) {
      int v = q[h++];
      if (level[v] > level[far] || (level[v] == level[far] && deg[v] < deg[far])) far = v;
      for (int p = m.ia[v]; p < m.ia[v + 1]; p++) {
        int w = m.ja[p];
        if (level[w] < 0) { level[w] = level[v] + 1; q.push_back(w); touched.push_back(w); }
      }
    }
    for (int v : touched) level[v] = -1;
    return far;
  };
  std::vector<int> nb;
  for (int s0 = 0; s0 < n; s0++) {
    if (seen[s0]) continue;
    int s = bfs_far(bfs_far(s0));
    size_t h = order.size();
    order.push_back(s);
    seen[s] = 1;
    while (h < order.size()) {
      int v = order[h++];
      nb.clear();
      for (int p = m.ia[v]; p < m.ia[v + 1]; p++) {
        int w = m.ja[p];
        if (!seen[w]) { seen[w] = 1; nb.push_back(w); }
      }
      std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  std::vector<int> new_of_old(n);
  for (int k = 0; k < n; k++) new_of_old[order[n - 1 - k]] = k;
  return new_of_old;
}

bool use_morton() {
  const char* e = std::getenv("SWE_ORDER");
  return !(e && std::string(e) == "rcm");
}

// Z-order (Morton) numbering of the nodes by their coordinates: 16-bit
// quantised x and y interleaved, ties broken by node index.  Consecutive rows
// form compact 2D patches, so the 32 rows of a warp gather neighbours that
// mostly share cache lines (an RCM level is a thin strip whose neighbours sit
// a bandwidth away); measured 3% faster per step than RCM on GB300, and the
// sort costs half of the BFS.
std::vector<int> morton_order(const HostMesh& m) {
  const int n = m.np;
  double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
  for (int i = 0; i < n; i++) {
    x0 = std::min(x0, m.rr[2 * (size_t)i]); x1 = std::max(x1, m.rr[2 * (size_t)i]);
    y0 = std::min(y0, m.rr[2 * (size_t)i + 1]); y1 = std::max(y1, m.rr[2 * (size_t)i + 1]);
  }
  const double sx = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, sy = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
  auto spread = [](uint32_t v) {
    uint64_t x = v & 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
  };
  // Hilbert index of (x, y) on a 2^16 grid (the classic rotate-and-flip
  // walk from the top bit down)
  auto hilbert = [](uint32_t x, uint32_t y) {
    uint64_t d = 0;
    for (uint32_t sq = 1u << 15; sq > 0; sq >>= 1) {
      const uint32_t rx = (x & sq) ? 1u : 0u, ry = (y & sq) ? 1u : 0u;
      d += (uint64_t)sq * sq * ((3u * rx) ^ ry);
      if (ry == 0) {
        if (rx == 1) { x = 0xffffu - x; y = 0xffffu - y; }
        const uint32_t t = x; x = y; y = t;
      }
    }
    return d;
  };
  const char* ord = std::getenv("SWE_ORDER");
  const bool hil = ord && std::string(ord) == "hilbert";
  std::vector<uint64_t> key(n);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    const uint32_t qx = (uint32_t)((m.rr[2 * (size_t)i] - x0) * sx), qy = (uint32_t)((m.rr[2 * (size_t)i + 1] - y0) * sy);
    key[i] = ((hil ? hilbert(qx, qy) : (spread(qx) | (spread(qy) << 1))) << 32) | (uint64_t)i;
  }
  std::sort(key.begin(), key.end());
  std::vector<int> out(n);
  for (int k = 0; k < n; k++) out[(int)(key[k] & 0xffffffffu)] = k;
  return out;
}

int sigma_rows() {
  const char* e = std::getenv("SWE_SIGMA");
  if (e) {
    const int v = std::atoi(e);
    if (v >= 0) return v;
  }
  return kSigmaRows;
}

// Within consecutive windows of `sigma` rows of an ordering, rows sorted by
// decreasing length (stable).  A SELL-32 slice then holds rows of nearly
// equal length, so its warp idles on few padded entries (on jittered
// Delaunay meshes the fill of the RCM order alone is ~77%, 96% with 256-row
// windows, 99% with 1024), while neighbours stay within the bandwidth plus
// one window of each other.  sigma = 0 keeps the ordering.
std::vector<int> sigma_sort(const HostMesh& m, const std::vector<int>& new_of_old, int sigma) {
  if (sigma <= 1) return new_of_old;
  const int n = m.np;
  std::vector<int> old_at(n);
  for (int i = 0; i < n; i++) old_at[new_of_old[i]] = i;
  for (int w0 = 0; w0 < n; w0 += sigma) {
    const int w1 = std::min(n, w0 + sigma);
    std::stable_sort(old_at.begin() + w0, old_at.begin() + w1,
                     [&](int a, int b) { return m.ia[a + 1] - m.ia[a] > m.ia[b + 1] - m.ia[b]; });
  }
  std::vector<int> out(n);
  for (int k = 0; k < n; k++) out[old_at[k]] = k;
  return out;
}

Layout build_layout(const std::vector<HostMesh>& meshes, const std::vector<std::vector<double>>& baths) {
  Layout L;
  L.n_inst = (int)meshes.size();
  L.row_off.assign(L.n_inst + 1, 0);
  for (int b = 0; b < L.n_inst; b++) {
    int64_t np = meshes[b].np;
    L.row_off[b + 1] = L.row_off[b] + (np + 31) / 32 * 32;
  }
  L.n_rows = L.row_off[L.n_inst];
  L.n_slices = L.n_rows / 32;
  L.len.assign(L.n_rows, 0);
  L.dpos.assign(L.n_rows, 0);
  L.valid.assign(L.n_rows, 0);
  L.cxii.assign(L.n_rows, 0.0);
  L.cyii.assign(L.n_rows, 0.0);
  L.ref_pos_diag.assign(L.n_rows, -1);
  L.lumped.assign(L.n_rows, 1.0);
  L.bath.assign(L.n_rows, 0.0);
  L.old_of_new.assign(L.n_rows, -1);
  L.slice_inst.assign(L.n_slices, 0);
  L.slice_w.assign(L.n_slices, 0);
  L.new_of_old.resize(L.n_inst);
  std::vector<std::vector<int>> nofs(L.n_inst);
#pragma omp parallel for schedule(dynamic)
  for (int b = 0; b < L.n_inst; b++)
    nofs[b] = sigma_sort(meshes[b], use_morton() ? morton_order(meshes[b]) : rcm_order(meshes[b]), sigma_rows());
  for (int b = 0; b < L.n_inst; b++) {
    const HostMesh& m = meshes[b];
    const std::vector<int>& nof = nofs[b];
    L.new_of_old[b].resize(m.np);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m.np; i++) {
      int64_t r = L.row_off[b] + nof[i];
      L.new_of_old[b][i] = (int)r;
      L.old_of_new[r] = i;
      L.len[r] = (uint8_t)(m.ia[i + 1] - m.ia[i] - 1);
      L.dpos[r] = (uint8_t)(m.diag[i] - m.ia[i]);
      L.valid[r] = 1;
      L.cxii[r] = m.cx[m.diag[i]];
      L.cyii[r] = m.cy[m.diag[i]];
      L.ref_pos_diag[r] = m.diag[i];
      L.lumped[r] = m.lumped[i];
      L.bath[r] = baths[b][i];
    }
    for (int64_t s = L.row_off[b] / 32; s < L.row_off[b + 1] / 32; s++) L.slice_inst[s] = b;
  }
  L.slice_ptr.assign(L.n_slices + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < L.n_slices; s++) {
    uint8_t w = 0;
    for (int l = 0; l < 32; l++) w = std::max(w, L.len[s * 32 + l]);
    L.slice_w[s] = w;
  }
  for (int64_t s = 0; s < L.n_slices; s++) L.slice_ptr[s + 1] = L.slice_ptr[s] + 32 * (int64_t)L.slice_w[s];
  L.n_entries = L.slice_ptr[L.n_slices];
  L.col.assign(L.n_entries, 0);
  L.cx.assign(L.n_entries, 0.0);
  L.cy.assign(L.n_entries, 0.0);
  L.ref_pos.assign(L.n_entries, -1);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < L.n_slices; s++)
    for (int l = 0; l < 32; l++) {
      int64_t r = s * 32 + l;
      for (int k = 0; k < L.slice_w[s]; k++) L.col[L.slice_ptr[s] + 32 * k + l] = (int)r;
    }
  for (int b = 0; b < L.n_inst; b++) {
    const HostMesh& m = meshes[b];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m.np; i++) {
      int64_t r = L.new_of_old[b][i];
      int64_t base = L.slice_ptr[r / 32] + (r % 32);
      int k = 0;
      for (int p = m.ia[i]; p < m.ia[i + 1]; p++) {
        if (p == m.diag[i]) continue;
        int64_t e = base + 32 * (int64_t)(k++);
        L.col[e] = L.new_of_old[b][m.ja[p]];
        L.cx[e] = m.cx[p];
        L.cy[e] = m.cy[p];
        L.ref_pos[e] = p;
      }
    }
  }
  return L;
}

bool build_row_tiles(const Layout& L, int tile, RowTiles& F) {
  if (tile <= 0 || tile % 32) return false;
  const int64_t n_tiles = (L.n_rows + tile - 1) / tile;
  F.tile = tile;
  F.loc.assign(L.n_entries, 0);
  F.halo_ptr.assign(n_tiles + 1, 0);
  std::vector<std::vector<int>> halo(n_tiles);
  bool ok = true;
#pragma omp parallel for schedule(dynamic, 64) reduction(&& : ok)
  for (int64_t t = 0; t < n_tiles; t++) {
    const int64_t r0 = t * tile, r1 = std::min<int64_t>(r0 + tile, L.n_rows);
    std::vector<int>& h = halo[t];
    for (int64_t r = r0; r < r1; r++) {
      const int64_t base = L.slice_ptr[r >> 5] + (r & 31);
      for (int k = 0; k < L.len[r]; k++) {
        const int j = L.col[base + 32 * k];
        if (j < r0 || j >= r1) h.push_back(j);
      }
    }
    std::sort(h.begin(), h.end());
    h.erase(std::unique(h.begin(), h.end()), h.end());
    if (tile + (int64_t)h.size() > 32767) ok = false;
    for (int64_t r = r0; r < r1; r++) {
      const int64_t base = L.slice_ptr[r >> 5] + (r & 31);
      for (int k = 0; k < L.len[r]; k++) {
        const int j = L.col[base + 32 * k];
        int pos = (int)(j - r0);
        if (j < r0 || j >= r1) pos = tile + (int)(std::lower_bound(h.begin(), h.end(), j) - h.begin());
        F.loc[base + 32 * k] = (int16_t)pos;
      }
    }
  }
  if (!ok) return false;
  F.halo_cap = 0;
  for (int64_t t = 0; t < n_tiles; t++) {
    F.halo_ptr[t + 1] = F.halo_ptr[t] + (int)halo[t].size();
    F.halo_cap = std::max(F.halo_cap, (int)halo[t].size());
  }
  F.halo_rows.resize(F.halo_ptr[n_tiles]);
  for (int64_t t = 0; t < n_tiles; t++) std::copy(halo[t].begin(), halo[t].end(), F.halo_rows.begin() + F.halo_ptr[t]);
  return true;
}

}  // namespace swe
