// fippi_cache.cu -- interoperable cache of the static near-pair integrals:
// the file format and the keys of the reference's FIPPI cache
// (FIPPICache.cc:126-400; PreloadCache / StoreCache, libscuff.h:662-663), so
// a cache written by either side warms the other's near field.
//
// A record is a search key of 15 floats (the canonically ordered vertices
// relative to the first one, each coordinate rounded to float before the
// subtraction, FIPPICache.cc:120-156) and the reference's QIFIPPIData: the
// 33 static integrals in its parametrisation (QIFIPPICubature.cc:187-330) plus
// the centroid x0 of the first panel.  This library keeps the same integrals in
// mesh vertex order with the monomials {1, u-v, v} and the cross moment
// relative to the first panel's vertex 0; the conversion is exact:
//  * each panel's canonical order is a permutation of its mesh order, and the
//    monomial bases of the two orders are related by a 3 x 3 matrix acting on
//    (1, b1, b2) (b = barycentrics of the mesh order);
//  * int int (x x x')/r^3 moves between origins with int int (x - x')/r^3;
//  * a flipped pair (the canonical order puts panel b first) transposes the
//    moments and negates both vector integrals.
// Process-wide, like the reference's GlobalFIPPICache: records preloaded from
// files, plus at store time the tables of every live geometry.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {

namespace {

struct RefFippi {  // QIFIPPIData (libscuffInternals.h:282-292)
  double xm[3], xx[3], rm1[9], r1[9], r2[9], x0[3];
};
static_assert(sizeof(RefFippi) == 288, "QIFIPPIData is 36 doubles");
constexpr size_t KEY_BYTES = 15 * sizeof(float);
constexpr size_t REC_BYTES = 64 + sizeof(RefFippi);  // key, padded to the doubles' alignment, then the data
const char SIGNATURE[] = "FIPPICACHE";                // written with its terminating zero

struct Key {
  float k[15];
  bool operator==(const Key& o) const { return memcmp(k, o.k, KEY_BYTES) == 0; }
};
struct KeyHash {
  size_t operator()(const Key& a) const {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the key bytes
    const unsigned char* p = (const unsigned char*)a.k;
    for (size_t i = 0; i < KEY_BYTES; i++) { h ^= p[i]; h *= 1099511628211ull; }
    return (size_t)h;
  }
};

std::mutex g_mu;
std::unordered_map<Key, RefFippi, KeyHash> g_table;
std::vector<Geometry*> g_live;

// "vertex less than" of AssessPanelPair.cc:250-266: coordinates compared in
// turn, each with a relative tolerance of 1e-6 of the first vertex's
// coordinate; equal vertices count as less
bool vlt(const double* a, const double* b) {
  for (int c = 0; c < 3; c++) {
    const double d = a[c] - b[c];
    if (std::fabs(d) > 1.0e-6 * std::fabs(a[c])) return d < 0.0;
  }
  return true;
}

// ascending order of three vertices by vlt, with the comparison sequence of
// CanonicallyOrderVertices (AssessPanelPair.cc:352-363)
void sort3(const double* const V[3], int o[3]) {
  int mn, md, mx;
  if (vlt(V[0], V[1])) { mn = 0; mx = 1; } else { mn = 1; mx = 0; }
  if (vlt(V[2], V[mn])) { md = mn; mn = 2; }
  else if (vlt(V[2], V[mx])) { md = 2; }
  else { md = mx; mx = 2; }
  o[0] = mn; o[1] = md; o[2] = mx;
}

// CanonicallyOrderVertices (AssessPanelPair.cc:342-455) for ncv = 0, 1, 2 on
// vertices in AssessPanelPair's order.  Returns whether the pair is flipped;
// the first canonical panel's slot k is vertex ia[k] of its panel, the
// second's ib[k] (panel b first when flipped).  For ncv = 0 both panels take
// panel a's sorted order and the flip test compares two vertices of panel a,
// exactly as the reference does: the keys must match its own.
bool canonical(int ncv, const double* const Va[3], const double* const Vb[3], int ia[3], int ib[3]) {
  if (ncv == 2) {
    const int a0 = vlt(Va[0], Va[1]) ? 0 : 1;
    ia[0] = ib[0] = a0; ia[1] = ib[1] = 1 - a0; ia[2] = ib[2] = 2;
    return !vlt(Va[2], Vb[2]);
  }
  if (ncv == 1) {
    const int a1 = vlt(Va[1], Va[2]) ? 1 : 2, b1 = vlt(Vb[1], Vb[2]) ? 1 : 2;
    const bool keep = vlt(Va[a1], Vb[b1]);
    const int pa[3] = {0, a1, 3 - a1}, pb[3] = {0, b1, 3 - b1};
    for (int k = 0; k < 3; k++) { ia[k] = keep ? pa[k] : pb[k]; ib[k] = keep ? pb[k] : pa[k]; }
    return !keep;
  }
  int oa[3], ob[3];
  sort3(Va, oa);
  sort3(Vb, ob);
  for (int k = 0; k < 3; k++) ia[k] = ib[k] = oa[k];
  return !vlt(Va[oa[0]], Va[ob[0]]);
}

// rows f = (1, u, v) of the canonical order as combinations of (1, b1, b2)
// of the mesh order; sig[k] = mesh vertex in canonical slot k.  With the TCR
// parametrisation x = V0 + u (V1 - V0) + v (V2 - V1) the barycentrics are
// (1 - u, u - v, v), so u = c1 + c2 and v = c2.
void basis_rows(const int sig[3], double R[3][3]) {
  auto bary = [](int m, double* r) {
    if (m == 0) { r[0] = 1.0; r[1] = -1.0; r[2] = -1.0; }
    else if (m == 1) { r[0] = 0.0; r[1] = 1.0; r[2] = 0.0; }
    else { r[0] = 0.0; r[1] = 0.0; r[2] = 1.0; }
  };
  double c1[3], c2[3];
  bary(sig[1], c1);
  bary(sig[2], c2);
  for (int j = 0; j < 3; j++) { R[0][j] = j == 0 ? 1.0 : 0.0; R[1][j] = c1[j] + c2[j]; R[2][j] = c2[j]; }
}

void inv3(const double A[3][3], double B[3][3]) {
  const double d = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                   A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  B[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / d;
  B[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / d;
  B[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / d;
  B[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / d;
  B[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / d;
  B[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / d;
  B[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / d;
  B[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / d;
  B[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / d;
}

// out = L M R^T for 3 x 3 matrices (M row-major, 9 doubles)
void sandwich(const double L[3][3], const double* M, const double R[3][3], double* out) {
  double t[9];
  for (int i = 0; i < 3; i++)
    for (int q = 0; q < 3; q++) {
      double s = 0.0;
      for (int p = 0; p < 3; p++) s += L[i][p] * M[3 * p + q];
      t[3 * i + q] = s;
    }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int q = 0; q < 3; q++) s += t[3 * i + q] * R[j][q];
      out[3 * i + j] = s;
    }
}

// everything the conversion of one near pair needs
struct PairMap {
  Key key;
  bool flipped;
  double Ra[3][3], Rb[3][3];  // canonical monomials of panels a and b over their mesh (1, b1, b2)
  double V0a[3];              // mesh vertex 0 of panel a (origin of this library's cross moment)
  double x0[3];               // centroid of the first canonical panel
};

void panel_vertices(const Geometry* g, int gp, double V[9]) {
  for (const Surface& S : g->S)
    if (gp >= S.panel_offset && gp < S.panel_offset + S.np) {
      const int p = gp - S.panel_offset;
      for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) V[3 * i + c] = S.V[3 * S.PV[3 * p + i] + c];
      return;
    }
}

void pair_map(const Geometry* g, const NearPair& n, PairMap* m) {
  double Va[9], Vb[9];
  panel_vertices(g, n.pa, Va);
  panel_vertices(g, n.pb, Vb);
  // AssessPanelPair's order: common vertices first (identity for ncv = 0)
  const double* Aa[3] = {Va + 3 * n.perm_a[0], Va + 3 * n.perm_a[1], Va + 3 * n.perm_a[2]};
  const double* Ab[3] = {Vb + 3 * n.perm_b[0], Vb + 3 * n.perm_b[1], Vb + 3 * n.perm_b[2]};
  int ia[3], ib[3];
  m->flipped = canonical(n.ncv, Aa, Ab, ia, ib);
  // mesh vertex in each canonical slot, per panel of this pair
  int sa[3], sb[3];
  const double *O1[3], *O2[3];
  for (int k = 0; k < 3; k++) {
    if (!m->flipped) {
      sa[k] = n.perm_a[ia[k]]; sb[k] = n.perm_b[ib[k]];
      O1[k] = Aa[ia[k]]; O2[k] = Ab[ib[k]];
    } else {
      sb[k] = n.perm_b[ia[k]]; sa[k] = n.perm_a[ib[k]];
      O1[k] = Ab[ia[k]]; O2[k] = Aa[ib[k]];
    }
  }
  basis_rows(sa, m->Ra);
  basis_rows(sb, m->Rb);
  for (int c = 0; c < 3; c++) {
    m->V0a[c] = Va[c];
    m->x0[c] = (O1[0][c] + O1[1][c] + O1[2][c]) / 3.0;
  }
  const double* rel[5] = {O1[1], O1[2], O2[0], O2[1], O2[2]};
  for (int q = 0; q < 5; q++)
    for (int c = 0; c < 3; c++) m->key.k[3 * q + c] = (float)rel[q][c] - (float)O1[0][c];
}

// this library's table entry (mesh order, monomials {1, u-v, v}) -> record
void to_ref(const PairMap& m, const Fippi& F, RefFippi* R) {
  // canonical monomials f = Ra g: M_f = Ra M_g Rb^T in this pair's order
  const double (*L)[3] = m.flipped ? m.Rb : m.Ra;
  const double (*Rr)[3] = m.flipped ? m.Ra : m.Rb;
  const double* src[3] = {F.RM1, F.R1, F.R2};
  double* dst[3] = {R->rm1, R->r1, R->r2};
  for (int t = 0; t < 3; t++) {
    double M[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) M[3 * i + j] = m.flipped ? src[t][3 * j + i] : src[t][3 * i + j];
    sandwich(L, M, Rr, dst[t]);
  }
  // absolute cross moment: (x - O) x (x' - O) = x x x' - (x - x') x O
  double xxa[3], xo[3];
  vcross(F.XM, m.V0a, xo);
  for (int c = 0; c < 3; c++) xxa[c] = F.XX[c] + xo[c];
  const double s = m.flipped ? -1.0 : 1.0;
  for (int c = 0; c < 3; c++) { R->xm[c] = s * F.XM[c]; R->xx[c] = s * xxa[c]; R->x0[c] = m.x0[c]; }
}

void from_ref(const PairMap& m, const RefFippi& R, Fippi* F) {
  double Li[3][3], Ri[3][3];
  inv3(m.flipped ? m.Rb : m.Ra, Li);
  inv3(m.flipped ? m.Ra : m.Rb, Ri);
  const double* src[3] = {R.rm1, R.r1, R.r2};
  double* dst[3] = {F->RM1, F->R1, F->R2};
  for (int t = 0; t < 3; t++) {
    double M[9];
    sandwich(Li, src[t], Ri, M);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) dst[t][3 * i + j] = m.flipped ? M[3 * j + i] : M[3 * i + j];
  }
  // keys are translation-free: the record may come from a copy of this pair
  // whose first panel sat at x0 (the correction of QDFIPPI.cc:143-158):
  // int int (x + d) x (x' + d) = x x x' + (x - x') x d
  double d[3], shift[3];
  for (int c = 0; c < 3; c++) d[c] = m.x0[c] - R.x0[c];
  vcross(R.xm, d, shift);
  const double s = m.flipped ? -1.0 : 1.0;
  double xo[3], xm[3];
  for (int c = 0; c < 3; c++) xm[c] = s * R.xm[c];
  vcross(xm, m.V0a, xo);
  for (int c = 0; c < 3; c++) { F->XM[c] = xm[c]; F->XX[c] = s * (R.xx[c] + shift[c]) - xo[c]; }
}

}  // namespace

// ---- library-internal hooks --------------------------------------------------
void cache_register(Geometry* g) {
  std::lock_guard<std::mutex> l(g_mu);
  g_live.push_back(g);
}
void cache_unregister(Geometry* g) {
  std::lock_guard<std::mutex> l(g_mu);
  for (size_t i = 0; i < g_live.size(); i++)
    if (g_live[i] == g) { g_live.erase(g_live.begin() + i); break; }
}
bool cache_active() {
  std::lock_guard<std::mutex> l(g_mu);
  return !g_table.empty();
}

// Fills table[i] for the block's near pairs found in the cache (ncv < 3) and
// lists the others in miss; returns the number of hits.
int cache_lookup(const Geometry* g, const Block& b, std::vector<Fippi>& table, std::vector<int>& miss) {
  table.assign(b.near.size(), Fippi());
  miss.clear();
  int hits = 0;
  std::lock_guard<std::mutex> l(g_mu);
  for (size_t i = 0; i < b.near.size(); i++) {
    const NearPair& n = b.near[i];
    if (n.ncv == 3) continue;
    PairMap m;
    pair_map(g, n, &m);
    auto it = g_table.find(m.key);
    if (it == g_table.end()) { miss.push_back((int)i); continue; }
    from_ref(m, it->second, &table[i]);
    hits++;
  }
  return hits;
}

// the same pair seen from panel b: its own common-vertices-first order (the
// reference evaluates pairs in both orders, and the canonical order of
// (b, a) need not be that of (a, b)), the moments transposed, the difference
// moment negated and the cross moment taken about panel b's vertex 0
static void swapped_pair(const Geometry* g, const NearPair& n, const Fippi& F, NearPair* ns, Fippi* Fs) {
  double Va[9], Vb[9];
  panel_vertices(g, n.pa, Va);
  panel_vertices(g, n.pb, Vb);
  *ns = n;
  ns->pa = n.pb;
  ns->pb = n.pa;
  const double* A[3] = {Vb, Vb + 3, Vb + 6};
  const double* B[3] = {Va, Va + 3, Va + 6};
  assess_pair(A, B, n.rmax, ns->perm_a, ns->perm_b);
  const double* src[3] = {F.RM1, F.R1, F.R2};
  double* dst[3] = {Fs->RM1, Fs->R1, Fs->R2};
  for (int t = 0; t < 3; t++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) dst[t][3 * j + i] = src[t][3 * i + j];
  // int x_a x x_b = XX + XM x V0a;  swapped: -(that) - (-XM) x V0b
  double xa[3], xb[3];
  vcross(F.XM, Va, xa);
  vcross(F.XM, Vb, xb);
  for (int c = 0; c < 3; c++) {
    Fs->XM[c] = -F.XM[c];
    Fs->XX[c] = -(F.XX[c] + xa[c]) + xb[c];
  }
}

static void insert_one(const Geometry* g, const NearPair& n, const Fippi& F) {
  PairMap m;
  pair_map(g, n, &m);
  if (g_table.count(m.key)) return;
  RefFippi R;
  to_ref(m, F, &R);
  g_table.emplace(m.key, R);
}

// adds a block's computed table to the cache, each pair in both orders
// (existing keys are kept)
static void cache_insert(const Geometry* g, const Block& b, const std::vector<Fippi>& table) {
  for (size_t i = 0; i < b.near.size(); i++) {
    const NearPair& n = b.near[i];
    if (n.ncv == 3 || n.pa == n.pb) continue;
    insert_one(g, n, table[i]);
    NearPair ns;
    Fippi Fs;
    swapped_pair(g, n, table[i], &ns, &Fs);
    insert_one(g, ns, Fs);
  }
}

void cache_stats(const Geometry* g, long long* hits, long long* misses) {
  *hits = *misses = 0;
  for (const Block& b : g->blocks) {
    std::vector<Fippi> table;
    std::vector<int> miss;
    *hits += cache_lookup(g, b, table, miss);
    *misses += (long long)miss.size();
  }
}

}  // namespace gbem

using namespace gbem;

extern "C" {

gbem_status gbem_cache_preload(const char* path) {
  if (!path) { set_error("gbem_cache_preload: NULL path"); return GBEM_EINVAL; }
  FILE* f = fopen(path, "rb");
  if (!f) { set_error("gbem_cache_preload: cannot open %s", path); return GBEM_EINVAL; }
  char sig[sizeof SIGNATURE];
  std::vector<unsigned char> rec(REC_BYTES);
  gbem_status st = GBEM_OK;
  if (fread(sig, sizeof sig, 1, f) != 1 || memcmp(sig, SIGNATURE, sizeof sig) != 0) {
    set_error("gbem_cache_preload: %s is not a FIPPI cache file", path);
    st = GBEM_EINVAL;
  } else {
    fseek(f, 0, SEEK_END);
    const long size = ftell(f) - (long)sizeof SIGNATURE;
    fseek(f, (long)sizeof SIGNATURE, SEEK_SET);
    if (size < 0 || size % (long)REC_BYTES != 0) {
      set_error("gbem_cache_preload: %s has an incorrect size", path);
      st = GBEM_EINVAL;
    } else {
      std::lock_guard<std::mutex> l(g_mu);
      for (long r = 0; r < size / (long)REC_BYTES; r++) {
        if (fread(rec.data(), REC_BYTES, 1, f) != 1) { set_error("gbem_cache_preload: short read"); st = GBEM_EINVAL; break; }
        Key k;
        RefFippi v;
        memcpy(k.k, rec.data(), KEY_BYTES);
        memcpy(&v, rec.data() + 64, sizeof v);
        g_table.emplace(k, v);
      }
    }
  }
  fclose(f);
  return st;
}

gbem_status gbem_cache_store(const char* path) {
  if (!path) { set_error("gbem_cache_store: NULL path"); return GBEM_EINVAL; }
  // tables of the live geometries whose near field has been computed
  std::vector<Geometry*> live;
  {
    std::lock_guard<std::mutex> l(g_mu);
    live = g_live;
  }
  for (Geometry* g : live) {
    if (!g->fippi_ready) continue;
    for (size_t bi = 0; bi < g->blocks.size(); bi++) {
      std::vector<Fippi> table;
      gbem_status st = download_fippi(g, bi, table);
      if (st != GBEM_OK) return st;
      std::lock_guard<std::mutex> l(g_mu);
      cache_insert(g, g->blocks[bi], table);
    }
  }
  FILE* f = fopen(path, "wb");
  if (!f) { set_error("gbem_cache_store: cannot open %s", path); return GBEM_EINVAL; }
  std::lock_guard<std::mutex> l(g_mu);
  bool ok = fwrite(SIGNATURE, sizeof SIGNATURE, 1, f) == 1;
  std::vector<unsigned char> rec(REC_BYTES, 0);
  for (const auto& kv : g_table) {
    if (!ok) break;
    memset(rec.data(), 0, REC_BYTES);
    memcpy(rec.data(), kv.first.k, KEY_BYTES);
    memcpy(rec.data() + 64, &kv.second, sizeof kv.second);
    ok = fwrite(rec.data(), REC_BYTES, 1, f) == 1;
  }
  fclose(f);
  if (!ok) { set_error("gbem_cache_store: write to %s failed", path); return GBEM_EINVAL; }
  return GBEM_OK;
}

gbem_status gbem_cache_clear(void) {
  std::lock_guard<std::mutex> l(g_mu);
  g_table.clear();
  return GBEM_OK;
}

gbem_status gbem_cache_size(long long* nrecords) {
  if (!nrecords) { set_error("gbem_cache_size: NULL argument"); return GBEM_EINVAL; }
  std::lock_guard<std::mutex> l(g_mu);
  *nrecords = (long long)g_table.size();
  return GBEM_OK;
}

}  // extern "C"
