// Mesh upload: the reference's Fortran mesh arrays -> colour-sorted sliced-ELL device layout.
//
// Replaces the per-call reads of type_mesh by solve_SSA (ice_dynamics_module.f90:607-661 walks
// colour_vi, CAaAc and the N*_AaAc coefficient columns; mesh_ArakawaC_module.f90:583-724 walks
// CAaAc for derivatives and the Neumann boundary) with one upload per mesh.
#include <algorithm>
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

void free_mesh(DevMesh &m) {
  void *ptrs[] = {m.orig_of_dev, m.dev_of_orig, m.deg, m.slice_ptr, m.col, m.cuv, m.nxy,
                  m.cuv32, m.nxy32, m.h_nxy, m.h_cuv, m.sNxy, m.s3Nxy, m.h_nxy32, m.s3Nxy32, m.bnd_ptr,
                  m.bnd_nbr, m.V, m.Aci12, m.iAci, m.nC};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  m = DevMesh();
}

}  // namespace

}  // namespace ufe

using namespace ufe;

extern "C" int ufe_mesh_create(const ufe_mesh_desc *d, ufe_mesh_h *out) {
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

  // Colour groups in colour_vi order (ascending row within a colour), edge rows removed.
  std::vector<int> colour_of(nA, -1);
  std::vector<std::vector<int>> groups(kGroups);
  int64_t total = 0;
  for (int c = 0; c < 5; ++c) {
    const int n_c = d->colour_nV[c];
    if (n_c < 0 || n_c > nA) { set_error("ufe_mesh_create: colour_nV out of range"); return UFE_BAD_MESH; }
    total += n_c;
    for (int k = 0; k < n_c; ++k) {
      const int r = d->colour_vi[k + (int64_t)c * nA] - 1;
      if (r < 0 || r >= nA || colour_of[r] >= 0) { set_error("ufe_mesh_create: colour_vi is not a partition"); return UFE_BAD_MESH; }
      colour_of[r] = c;
      if (!is_edge(r)) groups[c].push_back(r);
    }
  }
  if (total != nA) { set_error("ufe_mesh_create: colour_nV does not sum to nVAaAc"); return UFE_BAD_MESH; }
  // Host proof that each colour class is an independent set: the race-freedom of the
  // coloured sweep rests on it.
  for (int r = 0; r < nA; ++r)
    for (int c = 0; c < d->nCAaAc[r]; ++c)
      if (colour_of[CA(r, c)] == colour_of[r]) { set_error("ufe_mesh_create: two adjacent rows share a colour"); return UFE_BAD_MESH; }
  for (int c = 0; c < 5; ++c)
    std::stable_sort(groups[c].begin(), groups[c].end(),
                     [&](int a, int b) { return d->nCAaAc[a] > d->nCAaAc[b]; });
  for (int r = 4; r < nA; ++r)
    if (is_edge(r)) groups[5].push_back(r);
  const int n_edge = (int)groups[5].size();
  for (int r = 0; r < 4; ++r) groups[5].push_back(r);

  // ---- device row numbering -------------------------------------------------------------
  DevMesh m;
  m.nV = nV; m.nAc = nAc; m.nA = nA; m.ncm = ncm;
  int off = 0;
  for (int g = 0; g < kGroups; ++g) {
    m.grp_off[g] = off;
    m.grp_rows[g] = (int)groups[g].size();
    off += ((int)groups[g].size() + kSlice - 1) / kSlice * kSlice;
  }
  m.grp_off[kGroups] = off;
  m.nP = off;
  m.nSlices = off / kSlice;
  m.n_edge = n_edge;
  m.n_corner = 4;
  m.edge_first = m.grp_off[5];
  std::vector<int> orig_of_dev(m.nP, -1), dev_of_orig(nA, -1);
  for (int g = 0; g < kGroups; ++g)
    for (size_t k = 0; k < groups[g].size(); ++k) {
      orig_of_dev[m.grp_off[g] + k] = groups[g][k];
      dev_of_orig[groups[g][k]] = m.grp_off[g] + (int)k;
    }

  // ---- sliced ELL ------------------------------------------------------------------------
  std::vector<uint8_t> deg(m.nP, 0);
  std::vector<int64_t> slice_ptr(m.nSlices);
  int64_t nE = 0;
  for (int s = 0; s < m.nSlices; ++s) {
    int w = 0;
    for (int l = 0; l < kSlice; ++l) {
      const int r = orig_of_dev[s * kSlice + l];
      if (r >= 0) w = std::max(w, d->nCAaAc[r]);
    }
    slice_ptr[s] = nE;
    nE += (int64_t)w * kSlice;
  }
  m.nE = nE;
  for (int g = 0; g < kGroups; ++g) {
    const int sa = m.grp_off[g] / kSlice, sb = m.grp_off[g + 1] / kSlice;
    int prev_w = -1;
    for (int s = sa; s < sb; ++s) {
      const int w = (int)(((s + 1 < m.nSlices ? slice_ptr[s + 1] : nE) - slice_ptr[s]) / kSlice);
      if (w != prev_w) {
        if (m.n_runs[g] == kMaxRuns) { set_error("ufe_mesh_create: too many slice widths in a colour"); return UFE_BAD_MESH; }
        m.run_s0[g][m.n_runs[g]] = s;
        m.run_w[g][m.n_runs[g]] = w;
        m.run_e0[g][m.n_runs[g]] = slice_ptr[s];
        ++m.n_runs[g];
        prev_w = w;
      }
    }
  }
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

  // ---- Neumann boundary lists (apply_Neumann_boundary_AaAc) ------------------------------
  std::vector<int> bnd_ptr(1, 0), bnd_nbr;
  std::vector<int> edge_list_index(nA, -1);
  for (int k = 0; k < n_edge; ++k) edge_list_index[groups[5][k]] = k;
  for (int k = 0; k < n_edge; ++k) {
    const int r = groups[5][k];
    for (int c = 0; c < d->nCAaAc[r]; ++c) {
      const int j = CA(r, c);
      if (!is_edge(j)) bnd_nbr.push_back(dev_of_orig[j]);
    }
    if ((int)bnd_nbr.size() == bnd_ptr.back()) { set_error("ufe_mesh_create: edge row without non-edge neighbour"); return UFE_BAD_MESH; }
    bnd_ptr.push_back((int)bnd_nbr.size());
  }
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < d->nCAaAc[r]; ++c) {
      const int j = CA(r, c);
      if (j < 4) { set_error("ufe_mesh_create: corner connected to corner"); return UFE_BAD_MESH; }
      bnd_nbr.push_back(is_edge(j) ? -(edge_list_index[j] + 1) : dev_of_orig[j]);
    }
    bnd_ptr.push_back((int)bnd_nbr.size());
  }

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

  // ---- upload -------------------------------------------------------------------------------
  int dev = 0;
  int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return UFE_NO_DEVICE;
  ufe_mesh_s *h = new ufe_mesh_s();
  h->device = dev;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
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

extern "C" int ufe_mesh_destroy(ufe_mesh_h h) {
  if (!h) return UFE_OK;
  cudaStreamSynchronize(h->stream);
  ssa_free(h->ssa);
  sia_free(h->sia);
  free_mesh(h->m);
  cudaStreamDestroy(h->stream);
  delete h;
  return UFE_OK;
}

extern "C" void *ufe_mesh_stream(ufe_mesh_h h) { return h ? (void *)h->stream : nullptr; }
