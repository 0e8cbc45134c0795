// Mesh upload: the reference's Fortran mesh arrays -> colour-sorted sliced-ELL device layout.
//
// Replaces the per-call reads of type_mesh by solve_SSA (ice_dynamics_module.f90:607-661 walks
// colour_vi, CAaAc and the N*_AaAc coefficient columns; mesh_ArakawaC_module.f90:583-724 walks
// CAaAc for derivatives and the Neumann boundary) with one upload per mesh.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "ufe_internal.h"

namespace ufe {

namespace {

template <class T>
int dalloc(T **p, size_t n, const char *what) {
  if (n == 0) n = 1;
  return cuda_status(cudaMalloc((void **)p, n * sizeof(T)), what);
}

template <class T>
int upload(T **p, const std::vector<T> &h, cudaStream_t s, const char *what) {
  int rc = dalloc(p, h.size(), what);
  if (rc) return rc;
  if (h.empty()) return 0;
  return cuda_status(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), what);
}

// Host-only layout dump (tests): set by ufe_debug_dump_layout around a mesh_create that
// stops before touching the device and writes its host arrays to a file instead. Each record:
// a 32-byte name, an element-size byte, an element count (int64), the raw elements.
thread_local const char *t_dump_path = nullptr;
thread_local int t_dump_sms = 0;

struct LayoutDump {
  FILE *fp;
  bool good;
  explicit LayoutDump(const char *path) : fp(std::fopen(path, "wb")), good(fp != nullptr) {}
  ~LayoutDump() { if (fp) std::fclose(fp); }
  bool ok() const { return good; }
  template <class T>
  void put(const char *name, const std::vector<T> &v) {
    if (!good) return;
    char head[32] = {0};
    std::snprintf(head, sizeof head, "%s", name);
    const uint8_t es = (uint8_t)sizeof(T);
    const int64_t n = (int64_t)v.size();
    good = std::fwrite(head, 1, 32, fp) == 32 && std::fwrite(&es, 1, 1, fp) == 1 && std::fwrite(&n, 8, 1, fp) == 1 &&
           (n == 0 || std::fwrite(v.data(), sizeof(T), (size_t)n, fp) == (size_t)n);
  }
};

void free_mesh(DevMesh &m) {
  void *ptrs[] = {m.orig_of_dev, m.dev_of_orig, m.deg, m.slice_ptr, m.col, m.cuv, m.nxy,
                  m.cuv32, m.nxy32, m.h_nxy, m.h_cuv, m.sNxy, m.s3Nxy, m.h_nxy32, m.s3Nxy32, m.bnd_ptr,
                  m.bnd_nbr, m.V, m.Aci12, m.iAci, m.nC, m.patch_slice, m.patch_edge0, m.edge_row,
                  m.sync_ptr, m.sync_list, m.slice_e0, m.slice_w, m.slice_g, m.hp_slice, m.hp_split, m.hslice_e0,
                  m.hslice_w, m.hrow_l, m.hrow_g, m.hcol, m.hcuv32, m.hcuv, m.hload_ptr, m.hload_dev,
                  m.hsync_ptr, m.hsync_list, m.hs3_32, m.hs3};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  m = DevMesh();
}

// Slots of one phase of the halo sweep program: the phase's rows (device rows) dealt into
// slices of 32 lanes, densely (padding, -1, only after the last row). A slice's k-th gather
// reads, in each lane, the working-copy element (8 bytes in the mixed sweeps) of the lane's
// k-th neighbour; local index l lies in bank pair l mod 16, and the gather costs one
// shared-memory wavefront per element in its busiest bank pair (2 at best for 32 lanes, about 4.3
// in degree-sorted order on a 200k-vertex mesh). Rows are taken by degree, descending (stable):
// each slice starts with the first row not yet placed, so its width and the number of slices are
// those of plain degree order, and every next lane takes, among the next kWindow rows not yet
// placed, the one that raises the slice's per-entry maximum bank load least (the earliest on a
// tie). cols_of(p, cols) writes the local columns of p's entries and returns their number.
template <class ColsOf>
void bank_aware_slices(std::vector<int> &rows, ColsOf cols_of) {
  constexpr int kWindow = 64;
  const size_t n = rows.size();
  std::vector<int> nc(n), cols(n * kMaxDeg);
  for (size_t i = 0; i < n; ++i) nc[i] = cols_of(rows[i], &cols[i * kMaxDeg]);
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return nc[x] > nc[y]; });
  std::vector<char> used(n, 0);
  std::vector<int> out;
  out.reserve(n + kSlice);
  size_t first = 0;
  for (;;) {
    while (first < n && used[idx[first]]) ++first;
    if (first == n) break;
    int cnt[kMaxDeg][16], mx[kMaxDeg];
    std::memset(cnt, 0, sizeof cnt);
    std::memset(mx, 0, sizeof mx);
    auto take = [&](int i) {
      used[i] = 1;
      out.push_back(rows[i]);
      for (int k = 0; k < nc[i]; ++k) {
        int &c = cnt[k][cols[(size_t)i * kMaxDeg + k] & 15];
        if (++c > mx[k]) mx[k] = c;
      }
    };
    take(idx[first]);
    for (int lane = 1; lane < kSlice; ++lane) {
      int best = -1, best_cost = kMaxDeg + 1, seen = 0;
      for (size_t q = first + 1; q < n && seen < kWindow; ++q) {
        const int i = idx[q];
        if (used[i]) continue;
        ++seen;
        int c = 0;
        for (int k = 0; k < nc[i]; ++k) c += cnt[k][cols[(size_t)i * kMaxDeg + k] & 15] >= mx[k];
        if (c < best_cost) {
          best_cost = c;
          best = i;
          if (c == 0) break;
        }
      }
      if (best < 0) break;
      take(best);
    }
    while (out.size() % kSlice) out.push_back(-1);
  }
  rows.swap(out);
}

}  // namespace

}  // namespace ufe

using namespace ufe;

namespace ufe {

int mesh_create(const ufe_mesh_desc *d, int n_patch_request, ufe_mesh_h *out) {
  if (!d || !out) { set_error("ufe_mesh_create: null argument"); return UFE_BAD_ARG; }
  *out = nullptr;
  const int nV = d->nV, nAc = d->nAc, nA = d->nVAaAc, ncm = d->nC_mem;
  if (nV < 5 || nAc < 1 || nA != nV + nAc || ncm < 3 || ncm >= kMaxDeg) {
    set_error("ufe_mesh_create: inconsistent sizes (need nVAaAc = nV + nAc, 3 <= nC_mem < 32)");
    return UFE_BAD_ARG;
  }
  if (!d->V || !d->nC || !d->iAci || !d->Aci || !d->edge_index || !d->edge_index_Ac || !d->nCAaAc ||
      !d->CAaAc || !d->Nx_AaAc || !d->Ny_AaAc || !d->Nxx_AaAc || !d->Nxy_AaAc || !d->Nyy_AaAc ||
      !d->colour_vi || !d->colour_nV) {
    set_error("ufe_mesh_create: missing mesh array");
    return UFE_BAD_ARG;
  }
  // ---- classify rows and validate (before touching the device) ------------------------------------------------------
  auto is_edge = [&](int r) { return r < nV ? d->edge_index[r] > 0 : d->edge_index_Ac[r - nV] > 0; };
  auto CA = [&](int r, int c) { return d->CAaAc[r + (int64_t)c * nA] - 1; };
  for (int r = 0; r < nA; ++r) {
    const int n = d->nCAaAc[r];
    if (n < 2 || n > ncm) { set_error("ufe_mesh_create: nCAaAc out of range"); return UFE_BAD_MESH; }
    for (int c = 0; c < n; ++c) {
      const int j = CA(r, c);
      if (j < 0 || j >= nA || j == r) { set_error("ufe_mesh_create: CAaAc entry out of range"); return UFE_BAD_MESH; }
    }
  }
  for (int k = 0; k < 4; ++k)
    if (!is_edge(k)) { set_error("ufe_mesh_create: vertices 1..4 must be the domain corners"); return UFE_BAD_MESH; }

  // Colours (colour_vi lists), validated as a partition of the rows.
  std::vector<int> colour_of(nA, -1);
  int64_t total = 0;
  for (int c = 0; c < 5; ++c) {
    const int n_c = d->colour_nV[c];
    if (n_c < 0 || n_c > nA) { set_error("ufe_mesh_create: colour_nV out of range"); return UFE_BAD_MESH; }
    total += n_c;
    for (int k = 0; k < n_c; ++k) {
      const int r = d->colour_vi[k + (int64_t)c * nA] - 1;
      if (r < 0 || r >= nA || colour_of[r] >= 0) { set_error("ufe_mesh_create: colour_vi is not a partition"); return UFE_BAD_MESH; }
      colour_of[r] = c;
    }
  }
  if (total != nA) { set_error("ufe_mesh_create: colour_nV does not sum to nVAaAc"); return UFE_BAD_MESH; }
  // Host proof that each colour class is an independent set: the race-freedom of the
  // coloured sweep rests on it.
  for (int r = 0; r < nA; ++r)
    for (int c = 0; c < d->nCAaAc[r]; ++c)
      if (colour_of[CA(r, c)] == colour_of[r]) { set_error("ufe_mesh_create: two adjacent rows share a colour"); return UFE_BAD_MESH; }
  std::vector<int> edge_ord_of(nA, -1);   // filled below
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < d->nCAaAc[r]; ++c)
      if (CA(r, c) < 4) { set_error("ufe_mesh_create: corner connected to corner"); return UFE_BAD_MESH; }

  int dev = 0, num_sms = 0;
  int rc = UFE_OK;
  if (t_dump_path) {
    num_sms = t_dump_sms;   // host-only layout dump: no device is touched
  } else {
    rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (!rc) rc = cuda_status(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (rc || num_sms < 1) return UFE_NO_DEVICE;
  }

  // ---- spatial patches: one per CTA of the persistent solver ------------------------------
  // Rows in Morton order of their coordinates (Aa vertex, or the midpoint of the Ac edge),
  // cut into equal-count patches. Within a patch: the non-edge rows of colour 1..5, each
  // sorted by degree (stable in Morton order), then the patch's edge rows with corners last.
  // Every (patch, group) starts on a multiple of 32 rows.
  std::vector<double> xr(nA), yr(nA);
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for (int v = 0; v < nV; ++v) {
    xmin = std::min(xmin, d->V[v]); xmax = std::max(xmax, d->V[v]);
    ymin = std::min(ymin, d->V[v + (int64_t)nV]); ymax = std::max(ymax, d->V[v + (int64_t)nV]);
  }
  for (int r = 0; r < nA; ++r) {
    if (r < nV) { xr[r] = d->V[r]; yr[r] = d->V[r + (int64_t)nV]; continue; }
    const int a = r - nV;
    const int vi = d->Aci[a] - 1, vj = d->Aci[a + (int64_t)nAc] - 1;
    if (vi < 0 || vi >= nV || vj < 0 || vj >= nV) { set_error("ufe_mesh_create: Aci out of range"); return UFE_BAD_MESH; }
    xr[r] = 0.5 * (d->V[vi] + d->V[vj]);
    yr[r] = 0.5 * (d->V[vi + (int64_t)nV] + d->V[vj + (int64_t)nV]);
  }
  auto morton = [&](int r) {
    const double sx = xmax > xmin ? (xr[r] - xmin) / (xmax - xmin) : 0.0;
    const double sy = ymax > ymin ? (yr[r] - ymin) / (ymax - ymin) : 0.0;
    uint64_t ix = (uint64_t)std::min(65535.0, std::max(0.0, sx * 65536.0));
    uint64_t iy = (uint64_t)std::min(65535.0, std::max(0.0, sy * 65536.0));
    uint64_t k = 0;
    for (int b = 0; b < 16; ++b) k |= ((ix >> b) & 1u) << (2 * b) | ((iy >> b) & 1u) << (2 * b + 1);
    return k;
  };
  std::vector<uint64_t> key(nA);
  for (int r = 0; r < nA; ++r) key[r] = morton(r);
  std::vector<int> order(nA);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  // Default: one patch per CTA of the single-solve grid, at least kSsaBlock / 2 rows each. A
  // batched solve asks for its team size instead.
  const int n_patch = n_patch_request > 0 ? std::min(n_patch_request, std::max(1, nA / kSlice))
                                          : std::max(1, std::min(kCtasPerSm * num_sms, nA / (kSsaBlock / 2)));
  std::vector<int> patch_of(nA);
  std::vector<std::vector<std::vector<int>>> plist(n_patch, std::vector<std::vector<int>>(kGroups));
  for (int k = 0; k < nA; ++k) {
    const int r = order[k];
    const int b = (int)((int64_t)k * n_patch / nA);
    patch_of[r] = b;
    if (r < 4) continue;   // corners go last in their patch's edge group
    plist[b][is_edge(r) ? 5 : colour_of[r]].push_back(r);
  }
  for (int r = 0; r < 4; ++r) plist[patch_of[r]][5].push_back(r);
  for (int b = 0; b < n_patch; ++b)
    for (int g = 0; g < 5; ++g)
      std::stable_sort(plist[b][g].begin(), plist[b][g].end(),
                       [&](int x, int y) { return d->nCAaAc[x] > d->nCAaAc[y]; });

  // ---- device row numbering -------------------------------------------------------------
  DevMesh m;
  m.nV = nV; m.nAc = nAc; m.nA = nA; m.ncm = ncm; m.n_patch = n_patch;
  std::vector<int> patch_slice((size_t)n_patch * (kGroups + 1));
  std::vector<int> edge_row, patch_edge0(n_patch + 1, 0);
  int off = 0;
  for (int b = 0; b < n_patch; ++b) {
    for (int g = 0; g < kGroups; ++g) {
      patch_slice[(size_t)b * (kGroups + 1) + g] = off / kSlice;
      off += ((int)plist[b][g].size() + kSlice - 1) / kSlice * kSlice;
    }
    patch_slice[(size_t)b * (kGroups + 1) + kGroups] = off / kSlice;
  }
  m.nP = off;
  m.nSlices = off / kSlice;
  std::vector<int> orig_of_dev(m.nP, -1), dev_of_orig(nA, -1);
  std::vector<uint8_t> slice_g(m.nSlices, 255);
  int max_patch_slices = 0;
  for (int b = 0; b < n_patch; ++b) {
    for (int g = 0; g < kGroups; ++g) {
      const int p0 = patch_slice[(size_t)b * (kGroups + 1) + g] * kSlice;
      for (size_t k = 0; k < plist[b][g].size(); ++k) {
        orig_of_dev[p0 + k] = plist[b][g][k];
        dev_of_orig[plist[b][g][k]] = p0 + (int)k;
      }
      for (int s = patch_slice[(size_t)b * (kGroups + 1) + g]; s < patch_slice[(size_t)b * (kGroups + 1) + g + 1]; ++s)
        slice_g[s] = (uint8_t)g;
      if (g == 5) {
        patch_edge0[b] = (int)edge_row.size();
        for (size_t k = 0; k < plist[b][5].size(); ++k) {
          edge_ord_of[plist[b][5][k]] = (int)edge_row.size();
          edge_row.push_back(p0 + (int)k);
        }
        patch_edge0[b + 1] = (int)edge_row.size();
      }
    }
    max_patch_slices = std::max(max_patch_slices, patch_slice[(size_t)b * (kGroups + 1) + kGroups] -
                                                      patch_slice[(size_t)b * (kGroups + 1)]);
  }
  m.max_patch_slices = max_patch_slices;
  m.n_edge_total = (int)edge_row.size();
  if (max_patch_slices > kMaxPatchSlices) {
    set_error("ufe_mesh_create: a patch would hold more than 1024 slices of 32 rows (too few patches for this mesh)");
    return UFE_BAD_ARG;
  }

  // ---- sliced ELL ------------------------------------------------------------------------
  std::vector<uint8_t> deg(m.nP, 0);
  std::vector<int64_t> slice_ptr(m.nSlices);
  std::vector<uint8_t> slice_w(m.nSlices);
  int64_t nE = 0;
  for (int s = 0; s < m.nSlices; ++s) {
    int w = 0;
    for (int l = 0; l < kSlice; ++l) {
      const int r = orig_of_dev[s * kSlice + l];
      if (r >= 0) w = std::max(w, d->nCAaAc[r]);
    }
    slice_ptr[s] = nE;
    slice_w[s] = (uint8_t)w;
    nE += (int64_t)w * kSlice;
  }
  m.nE = nE;
  if (nE >= ((int64_t)1 << 31)) { set_error("ufe_mesh_create: more than 2^31 neighbour entries"); return UFE_BAD_ARG; }
  std::vector<int> slice_e0(m.nSlices);
  for (int s = 0; s < m.nSlices; ++s) slice_e0[s] = (int)slice_ptr[s];
  // padding entries (beyond a row's degree inside its slice) hold -1
  std::vector<int> col(nE, -1);
  std::vector<double2> cuv(nE, make_double2(0, 0)), nxy(nE, make_double2(0, 0));
  std::vector<float2> cuv32(nE, make_float2(0, 0)), nxy32(nE, make_float2(0, 0));
  std::vector<double2> h_nxy(m.nP, make_double2(0, 0)), h_cuv(m.nP, make_double2(0, 0));
  std::vector<double> sNxy(m.nP, 0.0), s3Nxy(m.nP, 0.0);
  std::vector<float2> h_nxy32(m.nP, make_float2(0, 0));
  std::vector<float> s3Nxy32(m.nP, 0.0f);
  const int64_t ldN = nA;
  auto N = [&](const double *a, int r, int c) { return a[r + (int64_t)c * ldN]; };
  for (int p = 0; p < m.nP; ++p) {
    const int r = orig_of_dev[p];
    if (r < 0) continue;
    const int n = d->nCAaAc[r];
    deg[p] = (uint8_t)n;
    const int s = p / kSlice, l = p % kSlice;
    double rsx = N(d->Nx_AaAc, r, n), rsy = N(d->Ny_AaAc, r, n), sxy = N(d->Nxy_AaAc, r, n);
    for (int c = 0; c < n; ++c) {
      const int64_t e = slice_ptr[s] + (int64_t)c * kSlice + l;
      const double nxx = N(d->Nxx_AaAc, r, c), nyy = N(d->Nyy_AaAc, r, c);
      col[e] = dev_of_orig[CA(r, c)];
      cuv[e] = make_double2(4.0 * nxx + nyy, 4.0 * nyy + nxx);
      nxy[e] = make_double2(N(d->Nx_AaAc, r, c), N(d->Ny_AaAc, r, c));
      cuv32[e] = make_float2((float)cuv[e].x, (float)cuv[e].y);
      nxy32[e] = make_float2((float)nxy[e].x, (float)nxy[e].y);
      rsx = rsx + nxy[e].x;
      rsy = rsy + nxy[e].y;
      sxy = sxy + N(d->Nxy_AaAc, r, c);
    }
    const double hxx = N(d->Nxx_AaAc, r, n), hyy = N(d->Nyy_AaAc, r, n);
    h_nxy[p] = make_double2(N(d->Nx_AaAc, r, n), N(d->Ny_AaAc, r, n));
    h_cuv[p] = make_double2(4.0 * hxx + hyy, 4.0 * hyy + hxx);
    sNxy[p] = sxy;
    s3Nxy[p] = 3.0 * sxy;
    h_nxy32[p] = make_float2((float)rsx, (float)rsy);
    s3Nxy32[p] = (float)(3.0 * sxy);
  }

  // ---- Neumann boundary lists (apply_Neumann_boundary_AaAc), by edge ordinal ------------
  // An edge row lists its non-edge neighbours; a corner lists all its neighbours, an edge
  // neighbour k encoded as -(k + 1) so that the corner recomputes that edge row's new value.
  std::vector<int> bnd_ptr(1, 0), bnd_nbr;
  std::vector<std::vector<int>> reads(n_patch);   // patches whose rows each patch reads
  for (int k = 0; k < m.n_edge_total; ++k) {
    const int r = orig_of_dev[edge_row[k]];
    const bool corner = r < 4;
    for (int c = 0; c < d->nCAaAc[r]; ++c) {
      const int j = CA(r, c);
      if (!is_edge(j)) {
        bnd_nbr.push_back(dev_of_orig[j]);
      } else if (corner) {
        bnd_nbr.push_back(-(edge_ord_of[j] + 1));
        for (int c2 = 0; c2 < d->nCAaAc[j]; ++c2)   // second-hop reads of the recompute
          if (!is_edge(CA(j, c2))) reads[patch_of[r]].push_back(patch_of[CA(j, c2)]);
      }
    }
    if ((int)bnd_nbr.size() == bnd_ptr.back()) { set_error("ufe_mesh_create: edge row without non-edge neighbour"); return UFE_BAD_MESH; }
    bnd_ptr.push_back((int)bnd_nbr.size());
  }
  m.bnd_total = (int)bnd_nbr.size();

  // ---- neighbour-patch synchronisation sets ------------------------------------------------
  // Patch b must not start a colour phase before every patch it reads from has finished the
  // previous phase, nor before every patch that reads from b has: the set is the symmetric
  // closure of the read relation (direct neighbours, plus the corners' second hop).
  for (int r = 0; r < nA; ++r)
    for (int c = 0; c < d->nCAaAc[r]; ++c) reads[patch_of[r]].push_back(patch_of[CA(r, c)]);
  std::vector<std::vector<int>> sync(n_patch);
  for (int b = 0; b < n_patch; ++b)
    for (int q : reads[b])
      if (q != b) { sync[b].push_back(q); sync[q].push_back(b); }
  std::vector<int> sync_ptr(1, 0), sync_list;
  int max_sync = 0;
  for (int b = 0; b < n_patch; ++b) {
    std::sort(sync[b].begin(), sync[b].end());
    sync[b].erase(std::unique(sync[b].begin(), sync[b].end()), sync[b].end());
    max_sync = std::max(max_sync, (int)sync[b].size());
    sync_list.insert(sync_list.end(), sync[b].begin(), sync[b].end());
    sync_ptr.push_back((int)sync_list.size());
  }
  m.max_sync = max_sync;
  if (max_sync > kMaxSync) { set_error("ufe_mesh_create: a patch touches too many other patches"); return UFE_BAD_MESH; }

  // ---- halo sweep program (single solves only) --------------------------------------------
  // Phases of a sweep: colours 0..4 (non-edge rows), 5 edge rows, 6 corners; an update reads
  // CAaAc neighbours (edge rows: the non-edge ones). A patch must also update every row of an
  // earlier phase that one of its updates reads (transitively): such a row is current only
  // after its own update in this sweep. Everything else it reads is a start-of-sweep value.
  std::vector<int> hp_slice, hp_split, hslice_e0, hrow_l, hrow_g, hload_ptr(1, 0), hload_dev, hsync_ptr(1, 0), hsync_list;
  std::vector<uint8_t> hslice_w;
  std::vector<uint16_t> hcol;
  std::vector<float2> hcuv32;
  std::vector<double2> hcuv;
  bool halo_ok = true;
  if (halo_ok) {
    std::vector<int8_t> ph(m.nP, -1);
    for (int p = 0; p < m.nP; ++p) {
      const int r = orig_of_dev[p];
      if (r >= 0) ph[p] = (int8_t)(r < 4 ? 6 : is_edge(r) ? 5 : colour_of[r]);
    }
    auto reads_of = [&](int p, std::vector<int> &out) {
      out.clear();
      const int r = orig_of_dev[p];
      for (int c = 0; c < d->nCAaAc[r]; ++c) {
        const int j = CA(r, c);
        if (ph[p] == 5 && is_edge(j)) continue;
        out.push_back(dev_of_orig[j]);
      }
    };
    std::vector<int> in_r(m.nP, -1), lidx(m.nP, -1), stamp(m.nP, -1), rd;
    std::vector<std::vector<int>> hreads(n_patch);
    int64_t nE_h = 0;
    for (int b = 0; b < n_patch && halo_ok; ++b) {
      const int p0 = patch_slice[(size_t)b * (kGroups + 1)] * kSlice;
      const int p1 = patch_slice[(size_t)b * (kGroups + 1) + kGroups] * kSlice;
      std::vector<int> R;
      for (int p = p0; p < p1; ++p)
        if (ph[p] >= 0) { in_r[p] = b; R.push_back(p); }
      for (size_t k = 0; k < R.size(); ++k) {
        reads_of(R[k], rd);
        for (int j : rd)
          if (ph[j] < ph[R[k]] && in_r[j] != b) { in_r[j] = b; R.push_back(j); }
      }
      // local slots: own device rows first, then the halo rows (every row read or updated)
      const int n_own = p1 - p0;
      std::vector<int> halo;
      auto local_of = [&](int p) {
        if (p >= p0 && p < p1) return p - p0;
        if (stamp[p] != b) { stamp[p] = b; lidx[p] = n_own + (int)halo.size(); halo.push_back(p); }
        return lidx[p];
      };
      for (int p : R) {
        local_of(p);
        reads_of(p, rd);
        for (int j : rd) local_of(j);
      }
      if (n_own + (int)halo.size() > 65535) { halo_ok = false; break; }
      m.max_local = std::max(m.max_local, n_own + (int)halo.size());
      m.max_halo = std::max(m.max_halo, (int)halo.size());
      for (int p : halo) hreads[b].push_back(patch_of[orig_of_dev[p]]);
      hload_dev.insert(hload_dev.end(), halo.begin(), halo.end());
      hload_ptr.push_back((int)hload_dev.size());
      // program: per phase, the phase's own and halo rows packed densely into slices of 32
      // (bank_aware_slices: by degree, lanes chosen to spread the working-copy gathers over
      // the shared-memory banks)
      const int first_slice = (int)hslice_e0.size();
      for (int f = 0; f < 7; ++f) {
        hp_slice.push_back((int)hslice_e0.size());
        std::vector<int> rows;   // device rows, -1 = padding slot
        for (int p = p0; p < p1; ++p)
          if (ph[p] == f) rows.push_back(p);
        for (int p : R)
          if ((p < p0 || p >= p1) && ph[p] == f) rows.push_back(p);
        auto cols_of = [&](int p, int *cols) {
          reads_of(p, rd);
          for (size_t k = 0; k < rd.size(); ++k) cols[k] = local_of(rd[k]);
          return (int)rd.size();
        };
        if (f == 0) {
          // colour 1's own rows that read no halo slot come first: a sweep runs them before it
          // waits for the neighbouring patches
          std::vector<int> early, late;
          for (int p : rows) {
            bool own_only = p >= p0 && p < p1;
            if (own_only) {
              reads_of(p, rd);
              for (int j : rd)
                if (local_of(j) >= n_own) { own_only = false; break; }
            }
            (own_only ? early : late).push_back(p);
          }
          bank_aware_slices(early, cols_of);
          bank_aware_slices(late, cols_of);
          hp_split.push_back((int)hslice_e0.size() + (int)(early.size() / kSlice));
          rows = early;
          rows.insert(rows.end(), late.begin(), late.end());
        } else {
          bank_aware_slices(rows, cols_of);
        }
        for (size_t s0 = 0; s0 < rows.size(); s0 += kSlice) {
          int w = 0;
          for (int l = 0; l < kSlice; ++l) {
            const int p = rows[s0 + l];
            if (p < 0) continue;
            reads_of(p, rd);
            w = std::max(w, (int)rd.size());
          }
          hslice_e0.push_back((int)nE_h);
          hslice_w.push_back((uint8_t)w);
          hcol.resize((size_t)nE_h + (size_t)w * kSlice, 0xffff);
          hcuv32.resize((size_t)nE_h + (size_t)w * kSlice, make_float2(0, 0));
          hcuv.resize((size_t)nE_h + (size_t)w * kSlice, make_double2(0, 0));
          for (int l = 0; l < kSlice; ++l) {
            const int p = rows[s0 + l];
            hrow_l.push_back(p < 0 ? -1 : local_of(p));
            hrow_g.push_back(p < 0 ? 0 : p);
            if (p < 0) continue;
            reads_of(p, rd);
            // the device SELL entries of p hold the same neighbours in the same order (the
            // edge rows' list skips their edge neighbours: their coefficients are unused)
            const int s = p / kSlice, ln = p % kSlice;
            for (size_t k = 0; k < rd.size(); ++k) {
              const size_t e = (size_t)nE_h + k * kSlice + l;
              hcol[e] = (uint16_t)local_of(rd[k]);
              if (f < 5) {
                const int64_t ed = slice_ptr[s] + (int64_t)k * kSlice + ln;
                hcuv32[e] = cuv32[ed];
                hcuv[e] = cuv[ed];
              }
            }
          }
          nE_h += (int64_t)w * kSlice;
        }
      }
      m.max_hslices = std::max(m.max_hslices, (int)hslice_e0.size() - first_slice);
      if (m.max_hslices > kMaxPatchSlices || nE_h >= ((int64_t)1 << 31)) halo_ok = false;
    }
    if (halo_ok) {
      hp_slice.push_back((int)hslice_e0.size());   // end of the last patch
      // the start-of-sweep wait: the owners of a patch's halo rows, and the patches that read it
      std::vector<std::vector<int>> hs(n_patch);
      for (int b = 0; b < n_patch; ++b)
        for (int q : hreads[b])
          if (q != b) { hs[b].push_back(q); hs[q].push_back(b); }
      for (int b = 0; b < n_patch; ++b) {
        std::sort(hs[b].begin(), hs[b].end());
        hs[b].erase(std::unique(hs[b].begin(), hs[b].end()), hs[b].end());
        m.max_hsync = std::max(m.max_hsync, (int)hs[b].size());
        hsync_list.insert(hsync_list.end(), hs[b].begin(), hs[b].end());
        hsync_ptr.push_back((int)hsync_list.size());
      }
      if (m.max_hsync > kMaxSync) halo_ok = false;
      m.n_hslices = (int)hslice_e0.size();
      m.n_hE = nE_h;
    }
  }
  m.has_halo = halo_ok;

  // ---- geometry ---------------------------------------------------------------------------
  std::vector<double2> V(nV);
  for (int v = 0; v < nV; ++v) V[v] = make_double2(d->V[v], d->V[v + (int64_t)nV]);
  std::vector<int2> Aci12(nAc);
  for (int a = 0; a < nAc; ++a) {
    Aci12[a] = make_int2(d->Aci[a] - 1, d->Aci[a + (int64_t)nAc] - 1);
    if (Aci12[a].x < 0 || Aci12[a].x >= nV || Aci12[a].y < 0 || Aci12[a].y >= nV) {
      set_error("ufe_mesh_create: Aci out of range");
      return UFE_BAD_MESH;
    }
  }
  std::vector<int> iAci((size_t)nV * ncm), nC(nV);
  for (int v = 0; v < nV; ++v) {
    nC[v] = d->nC[v];
    if (nC[v] < 2 || nC[v] > ncm) { set_error("ufe_mesh_create: nC out of range"); return UFE_BAD_MESH; }
    for (int c = 0; c < ncm; ++c) {
      const int a = d->iAci[v + (int64_t)c * nV] - 1;
      if (c < nC[v] && (a < 0 || a >= nAc)) { set_error("ufe_mesh_create: iAci out of range"); return UFE_BAD_MESH; }
      iAci[v + (size_t)c * nV] = c < nC[v] ? a : 0;
    }
  }

  if (t_dump_path) {
    LayoutDump f(t_dump_path);
    if (!f.ok()) { set_error("ufe_debug_dump_layout: cannot write the file"); return UFE_BAD_ARG; }
    const std::vector<int> sizes = {n_patch, m.nP, m.nSlices, m.max_local, m.has_halo ? 1 : 0, m.n_hslices, nA, nV};
    f.put("sizes", sizes);
    f.put("orig_of_dev", orig_of_dev); f.put("dev_of_orig", dev_of_orig); f.put("deg", deg);
    f.put("patch_slice", patch_slice); f.put("slice_ptr", slice_ptr); f.put("slice_w", slice_w); f.put("col", col);
    f.put("cuv", cuv); f.put("cuv32", cuv32); f.put("sync_ptr", sync_ptr); f.put("sync_list", sync_list);
    f.put("hp_slice", hp_slice); f.put("hp_split", hp_split); f.put("hslice_e0", hslice_e0); f.put("hslice_w", hslice_w);
    f.put("hrow_l", hrow_l); f.put("hrow_g", hrow_g); f.put("hcol", hcol); f.put("hcuv", hcuv);
    f.put("hcuv32", hcuv32); f.put("hload_ptr", hload_ptr); f.put("hload_dev", hload_dev);
    f.put("hsync_ptr", hsync_ptr); f.put("hsync_list", hsync_list);
    return f.ok() ? UFE_OK : UFE_BAD_ARG;
  }

  // ---- upload -------------------------------------------------------------------------------
  ufe_mesh_s *h = new ufe_mesh_s();
  h->device = dev;
  h->num_sms = num_sms;
  rc = cuda_status(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  auto S = h->stream;
  if (!rc) rc = upload(&m.orig_of_dev, orig_of_dev, S, "orig_of_dev");
  if (!rc) rc = upload(&m.dev_of_orig, dev_of_orig, S, "dev_of_orig");
  if (!rc) rc = upload(&m.deg, deg, S, "deg");
  if (!rc) rc = upload(&m.slice_ptr, slice_ptr, S, "slice_ptr");
  if (!rc) rc = upload(&m.col, col, S, "col");
  if (!rc) rc = upload(&m.cuv, cuv, S, "cuv");
  if (!rc) rc = upload(&m.nxy, nxy, S, "nxy");
  if (!rc) rc = upload(&m.cuv32, cuv32, S, "cuv32");
  if (!rc) rc = upload(&m.nxy32, nxy32, S, "nxy32");
  if (!rc) rc = upload(&m.h_nxy, h_nxy, S, "h_nxy");
  if (!rc) rc = upload(&m.h_cuv, h_cuv, S, "h_cuv");
  if (!rc) rc = upload(&m.sNxy, sNxy, S, "sNxy");
  if (!rc) rc = upload(&m.h_nxy32, h_nxy32, S, "h_nxy32");
  if (!rc) rc = upload(&m.s3Nxy, s3Nxy, S, "s3Nxy");
  if (!rc) rc = upload(&m.s3Nxy32, s3Nxy32, S, "s3Nxy32");
  if (!rc) rc = upload(&m.bnd_ptr, bnd_ptr, S, "bnd_ptr");
  if (!rc) rc = upload(&m.bnd_nbr, bnd_nbr, S, "bnd_nbr");
  if (!rc) rc = upload(&m.V, V, S, "V");
  if (!rc) rc = upload(&m.Aci12, Aci12, S, "Aci12");
  if (!rc) rc = upload(&m.iAci, iAci, S, "iAci");
  if (!rc) rc = upload(&m.nC, nC, S, "nC");
  if (!rc) rc = upload(&m.patch_slice, patch_slice, S, "patch_slice");
  if (!rc) rc = upload(&m.patch_edge0, patch_edge0, S, "patch_edge0");
  if (!rc) rc = upload(&m.edge_row, edge_row, S, "edge_row");
  if (!rc) rc = upload(&m.sync_ptr, sync_ptr, S, "sync_ptr");
  if (!rc) rc = upload(&m.sync_list, sync_list, S, "sync_list");
  if (!rc) rc = upload(&m.slice_e0, slice_e0, S, "slice_e0");
  if (!rc) rc = upload(&m.slice_w, slice_w, S, "slice_w");
  if (!rc) rc = upload(&m.slice_g, slice_g, S, "slice_g");
  if (!rc && m.has_halo) {
    rc = upload(&m.hp_slice, hp_slice, S, "hp_slice");
    if (!rc) rc = upload(&m.hp_split, hp_split, S, "hp_split");
    if (!rc) rc = upload(&m.hslice_e0, hslice_e0, S, "hslice_e0");
    if (!rc) rc = upload(&m.hslice_w, hslice_w, S, "hslice_w");
    if (!rc) rc = upload(&m.hrow_l, hrow_l, S, "hrow_l");
    if (!rc) rc = upload(&m.hrow_g, hrow_g, S, "hrow_g");
    if (!rc) rc = upload(&m.hcol, hcol, S, "hcol");
    if (!rc) rc = upload(&m.hcuv32, hcuv32, S, "hcuv32");
    if (!rc) rc = upload(&m.hcuv, hcuv, S, "hcuv");
    if (!rc) rc = upload(&m.hload_ptr, hload_ptr, S, "hload_ptr");
    if (!rc) rc = upload(&m.hload_dev, hload_dev, S, "hload_dev");
    if (!rc) rc = upload(&m.hsync_ptr, hsync_ptr, S, "hsync_ptr");
    if (!rc) rc = upload(&m.hsync_list, hsync_list, S, "hsync_list");
    // per-slot copies of the static cross-term coefficient (the kernels then need no
    // dependent load through the slot's device row)
    std::vector<float> hs3_32(hrow_g.size(), 0.0f);
    std::vector<double> hs3(hrow_g.size(), 0.0);
    for (size_t k = 0; k < hrow_g.size(); ++k)
      if (hrow_l[k] >= 0) { hs3_32[k] = s3Nxy32[hrow_g[k]]; hs3[k] = s3Nxy[hrow_g[k]]; }
    if (!rc) rc = upload(&m.hs3_32, hs3_32, S, "hs3_32");
    if (!rc) rc = upload(&m.hs3, hs3, S, "hs3");
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(S), "mesh upload");
  h->m = m;
  if (rc) {
    free_mesh(h->m);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return rc;
  }
  *out = h;
  return UFE_OK;
}

}  // namespace ufe

extern "C" int ufe_mesh_create(const ufe_mesh_desc *d, ufe_mesh_h *out) { return mesh_create(d, 0, out); }

// Test hook (not part of the public header): the device layout ufe_mesh_create would upload
// for a GPU of `num_sms` SMs, built on the host alone and written to `path` (record format
// in LayoutDump), so that its index arrays and the halo program can be checked without a GPU.
extern "C" int ufe_debug_dump_layout(const ufe_mesh_desc *d, int num_sms, int n_patch, const char *path) {
  if (!path || num_sms < 1) { set_error("ufe_debug_dump_layout: bad argument"); return UFE_BAD_ARG; }
  t_dump_path = path;
  t_dump_sms = num_sms;
  ufe_mesh_h h = nullptr;
  const int rc = mesh_create(d, n_patch, &h);
  t_dump_path = nullptr;
  return rc;
}

extern "C" int ufe_mesh_destroy(ufe_mesh_h h) {
  if (!h) return UFE_OK;
  cudaStreamSynchronize(h->stream);
  ssa_free(h->ssa);
  sia_free(h->sia);
  adj_free(h->adj);
  geom_free(h->geom);
  free_mesh(h->m);
  cudaStreamDestroy(h->stream);
  delete h;
  return UFE_OK;
}

extern "C" void *ufe_mesh_stream(ufe_mesh_h h) { return h ? (void *)h->stream : nullptr; }
