// geometry.cpp -- host-side mesh bookkeeping for the BEM hot path: panels,
// RWG edges, basis-function offsets, surface-pair blocks, edge tiles and the
// frequency-independent near-pair list.  Compiled with -ffp-contract=off so
// centroid/radius/relative-distance arithmetic rounds exactly like the
// reference's (the near/far branch choice depends on it).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include "gbem_internal.h"

namespace gbem {

static double dist3(const double* a, const double* b) {
  double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
  return std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

// Panel centroid and bounding radius (RWGSurface.cc:55-70).
static void init_panels(Surface& s) {
  s.cen.assign(3 * s.np, 0.0);
  s.rad.assign(s.np, 0.0);
  for (int p = 0; p < s.np; p++) {
    const double* v[3] = {&s.V[3 * s.PV[3 * p]], &s.V[3 * s.PV[3 * p + 1]], &s.V[3 * s.PV[3 * p + 2]]};
    double* c = &s.cen[3 * p];
    for (int i = 0; i < 3; i++) c[i] = (v[0][i] + v[1][i] + v[2][i]) / 3.0;
    double r = dist3(c, v[0]);
    r = std::fmax(r, dist3(c, v[1]));
    r = std::fmax(r, dist3(c, v[2]));
    s.rad[p] = r;
  }
}

// Interior RWG edges in the reference's order (InitEdgeList.cc:127-205):
// panels are walked in order, local edge j joins VI[j] and VI[j+1]; the first
// panel to visit an edge is its positive panel (Q = VI[j+2], PIndex = j+2),
// and the edge is numbered when the second panel visits it.
static gbem_status init_edges(Surface& s) {
  struct Rec { int v1, v2, qp, qm, pp, pm, pi, mi, idx; };
  std::vector<Rec> recs;
  recs.reserve(3 * s.np);
  std::unordered_map<long long, int> map;
  map.reserve(6 * s.np);
  int ne = 0;
  for (int p = 0; p < s.np; p++)
    for (int j = 0; j < 3; j++) {
      int a = s.PV[3 * p + j], b = s.PV[3 * p + (j + 1) % 3];
      int lo = std::min(a, b), hi = std::max(a, b);
      long long key = (long long)lo * (long long)(s.nv + 1) + hi;
      auto it = map.find(key);
      if (it == map.end()) {
        map.emplace(key, (int)recs.size());
        recs.push_back({lo, hi, s.PV[3 * p + (j + 2) % 3], -1, p, -1, (j + 2) % 3, (j + 2) % 3, -1});
      } else {
        Rec& r = recs[it->second];
        if (r.pm != -1) {
          set_error("invalid mesh topology: edge %d of panel %d also belongs to panels %d and %d", j, p, r.pp, r.pm);
          return GBEM_EMESH;
        }
        r.qm = s.PV[3 * p + (j + 2) % 3];
        r.pm = p;
        r.mi = (j + 2) % 3;
        r.idx = ne++;
      }
    }
  s.ne = ne;
  s.E.assign(8 * ne, 0);
  s.elen.assign(ne, 0.0);
  s.he_edge.assign(3 * s.np, -1);
  s.he_side.assign(3 * s.np, 0);
  for (const Rec& r : recs) {
    if (r.idx < 0) continue;  // exterior (half-RWG) edge: not a basis function
    int* e = &s.E[8 * r.idx];
    e[0] = r.v1; e[1] = r.v2; e[2] = r.qp; e[3] = r.qm; e[4] = r.pp; e[5] = r.pm; e[6] = r.pi; e[7] = r.mi;
    s.elen[r.idx] = dist3(&s.V[3 * r.v1], &s.V[3 * r.v2]);
    s.he_edge[3 * r.pp + r.pi] = r.idx; s.he_side[3 * r.pp + r.pi] = 0;
    s.he_edge[3 * r.pm + r.mi] = r.idx; s.he_side[3 * r.pm + r.mi] = 1;
  }
  return GBEM_OK;
}

// Greedy edge blocks: consecutive edges, at most TE edges and PMAX panels.
static std::vector<EdgeBlock> edge_blocks(const Surface& s) {
  std::vector<EdgeBlock> out;
  int e = 0;
  while (e < s.ne) {
    EdgeBlock b;
    b.e0 = e;
    std::vector<int> loc;  // surface panel -> local index
    std::unordered_map<int, int> pl;
    while (e < s.ne && b.ne < TE) {
      int pp = s.E[8 * e + 4], pm = s.E[8 * e + 5];
      int add = (pl.count(pp) ? 0 : 1) + (pm >= 0 && !pl.count(pm) && pm != pp ? 1 : 0);
      if ((int)pl.size() + add > PMAX) break;
      if (!pl.count(pp)) { pl[pp] = (int)b.panels.size(); b.panels.push_back(pp); }
      if (pm >= 0 && !pl.count(pm)) { pl[pm] = (int)b.panels.size(); b.panels.push_back(pm); }
      b.ne++;
      e++;
    }
    b.he_local.assign(3 * b.panels.size(), -1);
    b.he_side.assign(3 * b.panels.size(), 0);
    for (size_t i = 0; i < b.panels.size(); i++)
      for (int j = 0; j < 3; j++) {
        int ed = s.he_edge[3 * b.panels[i] + j];
        if (ed >= b.e0 && ed < b.e0 + b.ne) {
          b.he_local[3 * i + j] = (int8_t)(ed - b.e0);
          b.he_side[3 * i + j] = (int8_t)s.he_side[3 * b.panels[i] + j];
        }
      }
    for (auto& p : b.panels) p += s.panel_offset;
    out.push_back(std::move(b));
  }
  return out;
}

// Column stripes of a block (mixed far field): consecutive column edge blocks
// while the stripe's column panels times the row panels stay within a
// pair-value budget of STRIPE_PAIRS panel pairs (~0.5 GB of scratch at the
// largest field count); the row panels a stripe needs are those of the row
// edges up to its last column edge (a symmetric block keeps i <= j), or all.
constexpr size_t STRIPE_PAIRS = (size_t)3 << 20;

static void build_stripes(const Surface& sa, const Surface& sb, Block& blk) {
  blk.ecol.assign(sb.ne, make_int2(-1, -1));
  const int ncb = (int)blk.cols.size();
  // running maximum of the row panel index over the row edges
  std::vector<int> rowmax(sa.ne);
  int m = -1;
  for (int e = 0; e < sa.ne; e++) {
    m = std::max(m, std::max(sa.E[8 * e + 4], sa.E[8 * e + 5]));
    rowmax[e] = m;
  }
  int cb = 0;
  while (cb < ncb) {
    Stripe st;
    st.cb0 = cb;
    std::vector<char> in(sb.np, 0);
    size_t ncp = 0;
    while (cb < ncb) {
      const EdgeBlock& c = blk.cols[cb];
      size_t add = 0;
      std::vector<int> newp;
      for (int e = c.e0; e < c.e0 + c.ne; e++)
        for (int s = 0; s < 2; s++) {
          const int p = sb.E[8 * e + 4 + s];
          if (p >= 0 && !in[p]) { in[p] = 1; newp.push_back(p); add++; }
        }
      const int last = c.e0 + c.ne - 1;
      const size_t nrow = blk.sym ? (size_t)rowmax[std::min(last, sa.ne - 1)] + 1 : (size_t)sa.np;
      if (cb > st.cb0 && (ncp + add) * nrow > STRIPE_PAIRS) {
        for (int p : newp) in[p] = 0;
        break;
      }
      ncp += add;
      st.nrow = (int)nrow;
      cb++;
    }
    st.cb1 = cb;
    for (int p = 0; p < sb.np; p++)
      if (in[p]) st.cpan.push_back(p);
    std::vector<int> loc(sb.np, -1);
    for (size_t i = 0; i < st.cpan.size(); i++) loc[st.cpan[i]] = (int)i;
    for (int j = st.cb0; j < st.cb1; j++) {
      const EdgeBlock& c = blk.cols[j];
      for (int e = c.e0; e < c.e0 + c.ne; e++) {
        const int pp = sb.E[8 * e + 4], pm = sb.E[8 * e + 5];
        blk.ecol[e] = make_int2(pp >= 0 ? loc[pp] : -1, pm >= 0 ? loc[pm] : -1);
      }
      for (int i = 0; i < (int)blk.rows.size() && (!blk.sym || i <= j); i++) st.tiles.push_back(make_int2(i, j));
    }
    blk.max_stripe_pairs = std::max(blk.max_stripe_pairs, (size_t)st.nrow * st.cpan.size());
    blk.stripes.push_back(std::move(st));
  }
}

// Common-vertex count and common-vertices-first ordering
// (AssessPanelPair.cc:52-103; vertices within 1e-6 r_max count as common,
// VecClose of libs/libhrutil/Vector.cc:294-297).
static int assess(const double* Va[3], const double* Vb[3], double rmax, int8_t pa[3], int8_t pb[3]) {
  int ncv = 0, ca[3] = {0, 0, 0}, cb[3] = {0, 0, 0};
  double tol = std::fabs(1.0e-6 * rmax);
  for (int ia = 0; ia < 3; ia++)
    for (int ib = 0; ib < 3; ib++) {
      double d = std::fabs(Va[ia][0] - Vb[ib][0]) + std::fabs(Va[ia][1] - Vb[ib][1]) + std::fabs(Va[ia][2] - Vb[ib][2]);
      if (d <= 3 * tol && ncv < 3) { ca[ncv] = ia; cb[ncv] = ib; ncv++; }
    }
  for (int i = 0; i < 3; i++) { pa[i] = (int8_t)i; pb[i] = (int8_t)i; }
  if (ncv == 1) {
    for (int i = 0; i < 3; i++) { pa[i] = (int8_t)((ca[0] + i) % 3); pb[i] = (int8_t)((cb[0] + i) % 3); }
  } else if (ncv == 2) {
    pa[0] = ca[0]; pa[1] = ca[1]; pa[2] = 3 - ca[0] - ca[1];
    pb[0] = cb[0]; pb[1] = cb[1]; pb[2] = 3 - cb[0] - cb[1];
  } else if (ncv == 3) {
    for (int i = 0; i < 3; i++) { pa[i] = ca[i]; pb[i] = cb[i]; }
  }
  return ncv;
}

int assess_pair(const double* Va[3], const double* Vb[3], double rmax, int8_t pa[3], int8_t pb[3]) {
  return assess(Va, Vb, rmax, pa, pb);
}

// rRel exactly as AssessPanelPair.cc:160-166 computes it
static double rrel_of(const double* ca, const double* cb, double rmax) {
  double DC, r2;
  DC = ca[0] - cb[0]; r2 = DC * DC;
  DC = ca[1] - cb[1]; r2 += DC * DC;
  DC = ca[2] - cb[2]; r2 += DC * DC;
  return std::sqrt(r2) / rmax;
}

static void near_pairs(const Surface& A, const Surface& B, bool sym, Block& blk, long long* counts) {
  double rmaxg = 0;
  for (double r : A.rad) rmaxg = std::max(rmaxg, r);
  for (double r : B.rad) rmaxg = std::max(rmaxg, r);
  double h = 4.0 * rmaxg * 1.000001 + 1e-300;
  std::unordered_map<long long, std::vector<int>> grid;
  auto cell = [&](const double* c, int* ijk) { for (int i = 0; i < 3; i++) ijk[i] = (int)std::floor(c[i] / h); };
  auto key = [](int i, int j, int k) { return ((long long)(i + 1048576) << 42) | ((long long)(j + 1048576) << 21) | (long long)(k + 1048576); };
  for (int p = 0; p < B.np; p++) {
    int c[3]; cell(&B.cen[3 * p], c);
    grid[key(c[0], c[1], c[2])].push_back(p);
  }
  for (int a = 0; a < A.np; a++) {
    int c[3]; cell(&A.cen[3 * a], c);
    for (int dx = -1; dx <= 1; dx++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dz = -1; dz <= 1; dz++) {
          auto it = grid.find(key(c[0] + dx, c[1] + dy, c[2] + dz));
          if (it == grid.end()) continue;
          for (int b : it->second) {
            if (sym && b < a) continue;
            double rmax = std::fmax(A.rad[a], B.rad[b]);
            double rr = rrel_of(&A.cen[3 * a], &B.cen[3 * b], rmax);
            if (rr > 4.0) continue;
            NearPair np;
            np.pa = a + A.panel_offset;
            np.pb = b + B.panel_offset;
            np.rmax = rmax;
            const double* Va[3] = {&A.V[3 * A.PV[3 * a]], &A.V[3 * A.PV[3 * a + 1]], &A.V[3 * A.PV[3 * a + 2]]};
            const double* Vb[3] = {&B.V[3 * B.PV[3 * b]], &B.V[3 * B.PV[3 * b + 1]], &B.V[3 * B.PV[3 * b + 2]]};
            np.ncv = rr > 2.0 ? 0 : assess(Va, Vb, rmax, np.perm_a, np.perm_b);
            if (rr > 2.0) for (int i = 0; i < 3; i++) { np.perm_a[i] = (int8_t)i; np.perm_b[i] = (int8_t)i; }
            counts[np.ncv]++;
            if (np.ncv == 1 || np.ncv == 2) blk.rmax_touch = std::max(blk.rmax_touch, rmax);
            blk.near.push_back(np);
          }
        }
  }
  std::sort(blk.near.begin(), blk.near.end(), [](const NearPair& x, const NearPair& y) {
    return x.pa != y.pa ? x.pa < y.pa : x.pb < y.pb;
  });
  // CSR over row panels of surface A; entries (pb, index*2 + transposed)
  std::vector<std::vector<std::pair<int, int>>> rows(A.np);
  for (size_t i = 0; i < blk.near.size(); i++) {
    const NearPair& n = blk.near[i];
    rows[n.pa - A.panel_offset].push_back({n.pb, (int)(2 * i)});
    if (sym && n.pa != n.pb) rows[n.pb - A.panel_offset].push_back({n.pa, (int)(2 * i + 1)});
  }
  blk.near_ptr.assign(A.np + 1, 0);
  for (int a = 0; a < A.np; a++) {
    std::sort(rows[a].begin(), rows[a].end());
    blk.near_ptr[a + 1] = blk.near_ptr[a] + (int)rows[a].size();
  }
  for (int a = 0; a < A.np; a++)
    for (auto& pr : rows[a]) { blk.near_col.push_back(pr.first); blk.near_idx.push_back(pr.second); }
}

// Common regions of two surfaces and their relative signs
// (SurfaceSurfaceInteractions.cc:62-90).
static int common_regions(const Surface& a, const Surface& b, int reg[2], double sg[2]) {
  int n = 0;
  if (a.reg_ext == b.reg_ext) { reg[n] = a.reg_ext; sg[n] = 1.0; n++; }
  else if (a.reg_ext == b.reg_int) { reg[n] = a.reg_ext; sg[n] = -1.0; n++; }
  if (a.reg_int >= 0 && a.reg_int == b.reg_ext) { reg[n] = a.reg_int; sg[n] = -1.0; n++; }
  else if (!a.pec && !b.pec && a.reg_int == b.reg_int) { reg[n] = a.reg_int; sg[n] = 1.0; n++; }
  return n;
}

gbem_status build_geometry(int ns, const gbem_surface_desc* d, int nreg, Geometry* g) {
  if (ns <= 0 || !d || nreg <= 0) { set_error("gbem_geometry_create: bad arguments"); return GBEM_EINVAL; }
  g->nregions = nreg;
  g->S.resize(ns);
  int bf = 0, po = 0;
  for (int i = 0; i < ns; i++) {
    Surface& s = g->S[i];
    if (d[i].num_vertices <= 0 || d[i].num_panels <= 0 || !d[i].vertices || !d[i].panel_vertices) {
      set_error("surface %d: empty mesh", i);
      return GBEM_EINVAL;
    }
    if (d[i].exterior_region < 0 || d[i].exterior_region >= nreg || d[i].interior_region >= nreg ||
        (!d[i].is_pec && d[i].interior_region < 0)) {
      set_error("surface %d: bad region indices", i);
      return GBEM_EINVAL;
    }
    s.nv = d[i].num_vertices;
    s.np = d[i].num_panels;
    s.V.assign(d[i].vertices, d[i].vertices + 3 * s.nv);
    s.PV.assign(d[i].panel_vertices, d[i].panel_vertices + 3 * s.np);
    for (int v : s.PV)
      if (v < 0 || v >= s.nv) { set_error("surface %d: vertex index out of range", i); return GBEM_EINVAL; }
    s.reg_ext = d[i].exterior_region;
    s.reg_int = d[i].is_pec ? -1 : d[i].interior_region;
    s.pec = d[i].is_pec != 0;
    init_panels(s);
    gbem_status st = init_edges(s);
    if (st != GBEM_OK) return st;
    s.bf_offset = bf;
    s.panel_offset = po;
    bf += s.pec ? s.ne : 2 * s.ne;
    po += s.np;
  }
  g->N = bf;
  g->np_total = po;
  for (int a = 0; a < ns; a++)
    for (int b = a; b < ns; b++) {
      Block blk;
      blk.sa = a; blk.sb = b; blk.sym = (a == b);
      blk.nreg = common_regions(g->S[a], g->S[b], blk.reg, blk.sign);
      blk.bpe_a = g->S[a].pec ? 1 : 2;
      blk.bpe_b = g->S[b].pec ? 1 : 2;
      blk.rows = edge_blocks(g->S[a]);
      blk.cols = blk.sym ? blk.rows : edge_blocks(g->S[b]);
      for (int i = 0; i < (int)blk.rows.size(); i++)
        for (int j = blk.sym ? i : 0; j < (int)blk.cols.size(); j++) blk.tiles.push_back(make_int2(i, j));
      build_stripes(g->S[a], g->S[b], blk);
      if (blk.nreg > 0) near_pairs(g->S[a], g->S[b], blk.sym, blk, g->near_counts);
      g->blocks.push_back(std::move(blk));
    }
  return GBEM_OK;
}

}  // namespace gbem
