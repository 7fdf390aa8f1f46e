// Setup of the edge graph: the reference's construct_matrices
// (SOURCES/update.f90:18-132) on the device, then the GB300 layout (Morton or
// RCM renumbering, length-sorted SELL-32 slices) on the host.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace swe {

// One mesh in the caller's numbering, reference CSR order (0-based here).
struct HostMesh {
  int np = 0, me = 0;
  std::vector<int> jj;                   // (3, me), 0-based
  std::vector<double> rr;                // (2, np)
  std::vector<int> ia, ja;               // CSR, sorted columns, diagonal included
  std::vector<double> mass, cx, cy;      // per CSR entry
  std::vector<double> lumped;            // per node
  std::vector<int> diag;                 // CSR position of (i, i)
};

// Gauge location (condlim.f90:273-283): the first element m (0-based) for
// which inside(mesh, m, r) holds (SFEMaNS/FEMSUB_OBJET/post_interp.f90:
// 492-524), or -1; and the P1 weights FE_interpolation(mesh, m, r)
// (post_interp.f90:206-255) of the point in that element.
int gauge_element(const HostMesh& m, const double* r);
void gauge_weights(const HostMesh& m, int e, const double* r, double* ff);

// Builds ia/ja/mass/lumped/diag/cx/cy on the current CUDA device
// (swe_setup_gpu.cu) and copies them into m.  Returns "" or an error message.
std::string construct_matrices_device(HostMesh& m);

// Weights rj (3 per element) and points rr_gauss ((2, 3 me)) of the 3-point
// rule of gauss_points_2d_p1 (SFEMaNS/GAUSS_POINTS_OBJET/
// gauss_points_2d_p1.f90:95-128, 347-393); either may be null.
void gauss_points(const HostMesh& m, double* rj, double* rr_gauss);

// Reverse Cuthill-McKee ordering of the CSR graph: new_of_old[old] = new.
std::vector<int> rcm_order(const HostMesh& m);

// An ordering with rows sorted by decreasing length inside windows of sigma
// consecutive rows (SELL-C-sigma), new_of_old[old] = new.  sigma_rows() is
// kSigmaRows unless SWE_SIGMA sets it (0: plain RCM).
constexpr int kSigmaRows = 256;

// Z-order numbering by node coordinates, the default (SWE_ORDER=hilbert uses
// a Hilbert curve instead, SWE_ORDER=rcm RCM), new_of_old[old] = new.
std::vector<int> morton_order(const HostMesh& m);
bool use_morton();
int sigma_rows();
std::vector<int> sigma_sort(const HostMesh& m, const std::vector<int>& new_of_old, int sigma);

// Global SELL-32 layout of a batch of meshes (rows in Morton (or RCM) order,
// sorted by length within windows of sigma_rows()).  Row r (new numbering) of
// instance b lives in [row_off[b], row_off[b] + np_b); each instance's row
// range is padded to a multiple of 32 so that no slice straddles two
// instances.  Entry k of row r sits at slice_ptr[r/32] + 32*k + r%32.  The
// entries are the row's OFF-DIAGONAL CSR entries in reference order
// (ascending original column); the diagonal entry (i,i) is kept per row
// (cxii, cyii) together with dpos, the number of off-diagonal entries that
// precede it in the reference row, so that reference-order sums can insert it
// at its place.
struct Layout {
  int n_inst = 0;
  int64_t n_rows = 0;                    // padded total
  int64_t n_slices = 0;
  int64_t n_entries = 0;                 // padded total (multiple of 32)
  std::vector<int64_t> row_off;          // n_inst + 1
  std::vector<int64_t> slice_ptr;        // n_slices + 1, entry offsets
  std::vector<int> slice_inst;           // n_slices
  std::vector<uint8_t> slice_w;          // n_slices, max row length in slice
  std::vector<uint8_t> len;              // n_rows: off-diagonal entries (0 for padding rows)
  std::vector<uint8_t> dpos;             // n_rows: off-diagonal entries before the diagonal
  std::vector<uint8_t> valid;            // n_rows: 1 for mesh rows, 0 for padding rows
  std::vector<int> col;                  // n_entries (padding -> own row)
  std::vector<double> cx, cy;            // n_entries (padding -> 0)
  std::vector<double> cxii, cyii;        // n_rows: diagonal c_ii
  std::vector<int64_t> ref_pos;          // n_entries: instance-local CSR position or -1
  std::vector<int64_t> ref_pos_diag;     // n_rows: CSR position of (i,i) or -1
  std::vector<double> lumped, bath;      // n_rows
  std::vector<int64_t> old_of_new;       // n_rows: instance-local old index or -1
  std::vector<std::vector<int>> new_of_old;   // per instance, global row index
};

Layout build_layout(const std::vector<HostMesh>& meshes, const std::vector<std::vector<double>>& baths);

// Tiles of `tile` consecutive rows (a multiple of 32) for the shared-memory
// kernel variants.  halo_rows[halo_ptr[t] .. halo_ptr[t+1]) lists, ascending,
// the rows outside tile t that its entries reference; loc[e] is the column's
// position in the tile's shared-memory arrays: col - tile start for rows of
// the tile, tile + (index in the halo list) for halo rows, 0 for padding
// entries.  Returns false when a tile would need more than 32767 positions.
struct RowTiles {
  int tile = 0;
  int halo_cap = 0;
  std::vector<int16_t> loc;
  std::vector<int> halo_ptr, halo_rows;
};
bool build_row_tiles(const Layout& L, int tile, RowTiles& F);

}  // namespace swe
