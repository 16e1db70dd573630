// assemble.cu -- BEM matrix assembly on the GPU (replaces
// RWGGeometry::AssembleBEMMatrix, AssembleBEMMatrix.cc:684-765, and the
// GetSurfaceSurfaceInteractions / GetEdgeEdgeInteractions /
// GetPanelPanelInteractions stack below it for compact geometries).
//
// Kernels
//  fippi_kernel   once per geometry: the frequency-independent static
//                 integrals of every near panel pair (FP64).
//  self_kernel    per frequency: common-triangle pairs (FP64, Taylor-Duffy
//                 reduction to 1-D).
//  near_kernel    per frequency: every other pair with rRel <= 4 (FP64,
//                 desingularised 6x6 rule + static table, or high-order rule
//                 in the short-wavelength regime).
//  tile_kernel<T> per frequency: one CTA per tile of TE x TE edge pairs.
//                 Computes the 6x6-rule bilinear moments of every panel pair
//                 the tile touches once (T = float for the mixed form,
//                 double for the plain form), forms the up-to-9 (Qa,Qb)
//                 combinations, and writes the tile's matrix entries (and
//                 the mirrored tile) with coalesced stores.  Each edge-pair
//                 entry gathers its four panel-pair contributions from
//                 per-(edge pair, P/M side) slots in shared memory, so the
//                 sum is deterministic and needs no atomics.
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>
#include "adjoint.cuh"
#include "bem_math.cuh"
#include "ffmath.cuh"
#include "gbem_internal.h"

namespace gbem {

// ---------------------------------------------------------------------------
// quadrature rules in constant memory
// ---------------------------------------------------------------------------
// LO rule: the 13-digit values of libs/libTriInt/TCR.cc:83-91 (order 4).
__constant__ double c_lo64[18];
__constant__ FFRule c_ffrule;      // the LO rule as float-float (mixed far field)
__constant__ SinCosTab c_sctab;    // cos, sin of j pi/64 as float-float
static const double h_lo[18] = {
    0.0915762135098, 0.0915762135098, 0.0549758718276, 0.8168475729805, 0.0915762135098, 0.0549758718276,
    0.0915762135098, 0.8168475729805, 0.0549758718276, 0.1081030181681, 0.4459484909160, 0.1116907948390,
    0.4459484909160, 0.1081030181681, 0.1116907948390, 0.4459484909160, 0.4459484909160, 0.1116907948390};
constexpr int HO_N = 11;                 // collapsed Gauss rule, degree 20
__constant__ double c_ho[3 * HO_N * HO_N];
constexpr int NT_SELF = 16;              // 1-D rule of the common-triangle reduction
constexpr int N_FIP = 12;                // rules of the static near-pair integrals
__constant__ double c_gx16[NT_SELF], c_gw16[NT_SELF], c_gx12[N_FIP], c_gw12[N_FIP];
// static integrals inside the adjoint's central differences: 8 points per
// dimension move their derivatives by < 1e-8 (relative) against 12, at a
// third of the cost (touching pairs are the worst case)
constexpr int N_FIP_ADJ = 8;
__constant__ double c_gx8[N_FIP_ADJ], c_gw8[N_FIP_ADJ];

static void gauss01(int n, double* x, double* w) {
  for (int i = 0; i < n; i++) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double z1 = z;
      z = z1 - p1 / pp;
      if (fabs(z - z1) < 1e-16) break;
    }
    x[i] = 0.5 * (1 - z);
    w[i] = 1.0 / ((1 - z * z) * pp * pp);
  }
}

static gbem_status init_rules() {
  static bool done[64] = {false};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && done[dev]) return GBEM_OK;
  double x[HO_N], w[HO_N], ho[3 * HO_N * HO_N];
  gauss01(HO_N, x, w);
  int k = 0;
  for (int i = 0; i < HO_N; i++)
    for (int j = 0; j < HO_N; j++) {
      ho[k++] = x[i] * (1.0 - x[j]);
      ho[k++] = x[i] * x[j];
      ho[k++] = w[i] * w[j] * x[i];
    }
  double gx16[NT_SELF], gw16[NT_SELF], gx12[N_FIP], gw12[N_FIP];
  gauss01(NT_SELF, gx16, gw16);
  gauss01(N_FIP, gx12, gw12);
  double gx8[N_FIP_ADJ], gw8[N_FIP_ADJ];
  gauss01(N_FIP_ADJ, gx8, gw8);
  FFRule ffr;
  fill_ff_rule(h_lo, &ffr);
  SinCosTab sct;
  fill_sincos_tab(&sct);
  cudaError_t e = cudaMemcpyToSymbol(c_lo64, h_lo, sizeof h_lo);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ffrule, &ffr, sizeof ffr);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_sctab, &sct, sizeof sct);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ho, ho, sizeof ho);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gx16, gx16, sizeof gx16);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gw16, gw16, sizeof gw16);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gx12, gx12, sizeof gx12);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gw12, gw12, sizeof gw12);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gx8, gx8, sizeof gx8);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gw8, gw8, sizeof gw8);
  if (e != cudaSuccess) return cuda_status(e, "copy quadrature rules");
  if (dev < 64) done[dev] = true;
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// device-side geometry
// ---------------------------------------------------------------------------
struct DevEdgeBlock {
  int e0, ne, np, pad;
  int panels[PMAX];
  int8_t hl[3 * PMAX];
  int8_t hs[3 * PMAX];
};

struct DevNear {
  int pa, pb;
  int ncv;
  int perm_a[3], perm_b[3];  // common-vertices-first order -> mesh order
  double rmax;
};

struct DevBlock {
  int nrows = 0, ncols = 0, ntiles = 0, nnear = 0, nself = 0, nother = 0;
  DevEdgeBlock* rows = nullptr;
  DevEdgeBlock* cols = nullptr;
  int2* tiles = nullptr;
  double* elen_a = nullptr;
  double* elen_b = nullptr;
  int* nptr = nullptr;
  int* ncol = nullptr;
  int* nidx = nullptr;
  DevNear* near = nullptr;
  int* self_list = nullptr;
  int* other_list = nullptr;
  Fippi* fippi = nullptr;     // per near pair (unused slots for self pairs)
  double* nearval = nullptr;  // 27 complex per near pair
  // column stripes of the mixed far field
  struct DevStripe {
    int nrow = 0, ncp = 0, ntiles = 0;
    int* cpan = nullptr;
    int2* tiles = nullptr;
  };
  std::vector<DevStripe> stripes;
  int4* edge_a = nullptr;  // per row edge: P panel, its Q index, M panel, its Q index
  int4* edge_b = nullptr;  // per column edge, likewise
  int2* ecol = nullptr;    // per column edge: stripe-local P, M panel index
};

template <typename Tp>
static cudaError_t dupload(Tp** d, const Tp* h, size_t n) {
  if (n == 0) { *d = nullptr; return cudaSuccess; }
  cudaError_t e = cudaMalloc((void**)d, n * sizeof(Tp));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h, n * sizeof(Tp), cudaMemcpyHostToDevice);
}

static DevEdgeBlock pack_block(const EdgeBlock& b) {
  DevEdgeBlock d;
  memset(&d, 0, sizeof d);
  d.e0 = b.e0; d.ne = b.ne; d.np = (int)b.panels.size();
  for (int i = 0; i < d.np; i++) d.panels[i] = b.panels[i];
  for (int i = 0; i < 3 * d.np; i++) { d.hl[i] = b.he_local[i]; d.hs[i] = b.he_side[i]; }
  return d;
}

gbem_status upload_geometry(Geometry* g) {
  if (g->d_pv) return GBEM_OK;
  cudaError_t e = cudaSetDevice(g->device);
  if (e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
  gbem_status st = init_rules();
  if (st != GBEM_OK) return st;
  std::vector<double> pv(9 * (size_t)g->np_total), pc(4 * (size_t)g->np_total);
  for (const Surface& s : g->S)
    for (int p = 0; p < s.np; p++) {
      size_t gp = s.panel_offset + p;
      for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) pv[9 * gp + 3 * i + c] = s.V[3 * s.PV[3 * p + i] + c];
      for (int c = 0; c < 3; c++) pc[4 * gp + c] = s.cen[3 * p + c];
      pc[4 * gp + 3] = s.rad[p];
    }
  e = dupload(&g->d_pv, pv.data(), pv.size());
  if (e == cudaSuccess) e = dupload(&g->d_pc, pc.data(), pc.size());
  if (e != cudaSuccess) return cuda_status(e, "upload panels");
  for (const Block& b : g->blocks) {
    DevBlock* db = new DevBlock();
    g->dblocks.push_back(db);
    std::vector<DevEdgeBlock> rows, cols;
    for (auto& eb : b.rows) rows.push_back(pack_block(eb));
    for (auto& eb : b.cols) cols.push_back(pack_block(eb));
    db->nrows = (int)rows.size(); db->ncols = (int)cols.size(); db->ntiles = (int)b.tiles.size();
    e = dupload(&db->rows, rows.data(), rows.size());
    if (e == cudaSuccess) e = dupload(&db->cols, cols.data(), cols.size());
    if (e == cudaSuccess) e = dupload(&db->tiles, b.tiles.data(), b.tiles.size());
    if (e == cudaSuccess) e = dupload(&db->elen_a, g->S[b.sa].elen.data(), g->S[b.sa].elen.size());
    if (e == cudaSuccess) e = dupload(&db->elen_b, g->S[b.sb].elen.data(), g->S[b.sb].elen.size());
    if (e == cudaSuccess) e = dupload(&db->nptr, b.near_ptr.data(), b.near_ptr.size());
    if (e == cudaSuccess) e = dupload(&db->ncol, b.near_col.data(), b.near_col.size());
    if (e == cudaSuccess) e = dupload(&db->nidx, b.near_idx.data(), b.near_idx.size());
    std::vector<DevNear> dn;
    std::vector<int> self_l, other_l[3];
    for (size_t i = 0; i < b.near.size(); i++) {
      const NearPair& n = b.near[i];
      DevNear d;
      d.pa = n.pa; d.pb = n.pb; d.ncv = n.ncv; d.rmax = n.rmax;
      for (int j = 0; j < 3; j++) { d.perm_a[j] = n.perm_a[j]; d.perm_b[j] = n.perm_b[j]; }
      dn.push_back(d);
      if (n.ncv == 3) self_l.push_back((int)i); else other_l[n.ncv].push_back((int)i);
    }
    std::vector<int> others;
    for (int c = 0; c < 3; c++) others.insert(others.end(), other_l[c].begin(), other_l[c].end());
    db->nnear = (int)dn.size(); db->nself = (int)self_l.size(); db->nother = (int)others.size();
    if (e == cudaSuccess) e = dupload(&db->near, dn.data(), dn.size());
    if (e == cudaSuccess) e = dupload(&db->self_list, self_l.data(), self_l.size());
    if (e == cudaSuccess) e = dupload(&db->other_list, others.data(), others.size());
    if (e == cudaSuccess && db->nnear) e = cudaMalloc((void**)&db->fippi, sizeof(Fippi) * db->nnear);
    if (e == cudaSuccess && db->nnear) e = cudaMalloc((void**)&db->nearval, sizeof(double) * 54 * db->nnear);
    // edge tables and column stripes of the mixed far field
    auto edge4 = [](const Surface& S) {
      std::vector<int4> t(S.ne);
      for (int i = 0; i < S.ne; i++) t[i] = make_int4(S.E[8 * i + 4], S.E[8 * i + 6], S.E[8 * i + 5], S.E[8 * i + 7]);
      return t;
    };
    const std::vector<int4> ea = edge4(g->S[b.sa]), eb = edge4(g->S[b.sb]);
    if (e == cudaSuccess) e = dupload(&db->edge_a, ea.data(), ea.size());
    if (e == cudaSuccess) e = dupload(&db->edge_b, eb.data(), eb.size());
    if (e == cudaSuccess) e = dupload(&db->ecol, b.ecol.data(), b.ecol.size());
    for (const Stripe& st : b.stripes) {
      DevBlock::DevStripe ds;
      ds.nrow = st.nrow; ds.ncp = (int)st.cpan.size(); ds.ntiles = (int)st.tiles.size();
      if (e == cudaSuccess) e = dupload(&ds.cpan, st.cpan.data(), st.cpan.size());
      if (e == cudaSuccess) e = dupload(&ds.tiles, st.tiles.data(), st.tiles.size());
      db->stripes.push_back(ds);
    }
    if (e != cudaSuccess) return cuda_status(e, "upload blocks");
  }
  // float-float rule nodes and geometry of every panel, relative to the mean
  // vertex (the mixed far field's positions: ~48 bits relative to that origin)
  double O[3] = {0.0, 0.0, 0.0};
  for (size_t gp = 0; gp < (size_t)g->np_total; gp++)
    for (int c = 0; c < 3; c++) O[c] += (pv[9 * gp + c] + pv[9 * gp + 3 + c] + pv[9 * gp + 6 + c]) / (3.0 * g->np_total);
  std::vector<float> node(36 * (size_t)g->np_total), geo(18 * (size_t)g->np_total);
  for (size_t gp = 0; gp < (size_t)g->np_total; gp++) {
    const double* V = pv.data() + 9 * gp;
    double v0[3], A[3], B[3];
    for (int c = 0; c < 3; c++) { v0[c] = V[c] - O[c]; A[c] = V[3 + c] - V[c]; B[c] = V[6 + c] - V[c]; }
    for (int c = 0; c < 3; c++) {
      const ff x = ff_of(v0[c]), y = ff_of(A[c]), z = ff_of(B[c]);
      geo[18 * gp + c] = x.hi; geo[18 * gp + 3 + c] = x.lo;
      geo[18 * gp + 6 + c] = y.hi; geo[18 * gp + 9 + c] = y.lo;
      geo[18 * gp + 12 + c] = z.hi; geo[18 * gp + 15 + c] = z.lo;
    }
    for (int i = 0; i < 6; i++)
      for (int c = 0; c < 3; c++) {
        const ff x = ff_of(v0[c] + h_lo[3 * i] * A[c] + h_lo[3 * i + 1] * B[c]);
        node[36 * gp + 6 * i + c] = x.hi; node[36 * gp + 6 * i + 3 + c] = x.lo;
      }
  }
  e = dupload(&g->d_ffnode, node.data(), node.size());
  if (e == cudaSuccess) e = dupload(&g->d_ffgeo, geo.data(), geo.size());
  if (e != cudaSuccess) return cuda_status(e, "upload float-float panels");
  return GBEM_OK;
}

void free_geometry_device(Geometry* g) {
  cudaFree(g->d_pv); cudaFree(g->d_pc);
  g->d_pv = g->d_pc = nullptr;
  for (DevBlock* db : g->dblocks) {
    cudaFree(db->rows); cudaFree(db->cols); cudaFree(db->tiles); cudaFree(db->elen_a); cudaFree(db->elen_b);
    cudaFree(db->nptr); cudaFree(db->ncol); cudaFree(db->nidx); cudaFree(db->near); cudaFree(db->self_list);
    cudaFree(db->other_list); cudaFree(db->fippi); cudaFree(db->nearval);
    cudaFree(db->edge_a); cudaFree(db->edge_b); cudaFree(db->ecol);
    for (auto& st : db->stripes) { cudaFree(st.cpan); cudaFree(st.tiles); }
    delete db;
  }
  g->dblocks.clear();
  cudaFree(g->d_ffnode); cudaFree(g->d_ffgeo); cudaFree(g->ppv);
  cudaFree(g->d_pvi); cudaFree(g->d_sbf); cudaFree(g->d_ssl);
  g->d_pvi = g->d_sbf = nullptr;
  g->d_ssl = nullptr;
  g->d_ffnode = g->d_ffgeo = nullptr;
  g->ppv = nullptr;
  g->ppv_bytes = 0;
}

// ---------------------------------------------------------------------------
// per-frequency region data of a block
// ---------------------------------------------------------------------------
struct RegionArgs {
  int nreg;
  cx<double> k[2];     // wavenumber per common region
  cx<double> pf1[2];   // +-i mu omega   (SurfaceSurfaceInteractions.cc:165-176)
  cx<double> pfc[2];   // (-+i k) / (i k) : multiplies H1 (GC[1] carries 1/(ik))
  cx<double> pf3[2];   // -+i eps omega
};


// ---------------------------------------------------------------------------
// static near-pair table (once per geometry)
// ---------------------------------------------------------------------------
// One warp per near pair: the pair's cubature points are dealt to the lanes
// (lane l takes points l, l + 32, ...), each lane keeps its 33 partial sums
// in registers, and a shuffle reduction forms the pair's table entry.  The
// rule sits in shared memory (lanes read different nodes at once).
constexpr int FIPPI_THREADS = 128;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// every lane ends with the warp's totals
__device__ __forceinline__ void fippi_warp_sum(Fippi& F) {
#pragma unroll
  for (int m = 0; m < 9; m++) {
    F.RM1[m] = warp_sum(F.RM1[m]);
    F.R1[m] = warp_sum(F.R1[m]);
    F.R2[m] = warp_sum(F.R2[m]);
  }
#pragma unroll
  for (int m = 0; m < 3; m++) {
    F.XM[m] = warp_sum(F.XM[m]);
    F.XX[m] = warp_sum(F.XX[m]);
  }
}

__device__ __forceinline__ void cx_warp_sum(cx<double>* v, int n) {
  for (int m = 0; m < n; m++) { v[m].re = warp_sum(v[m].re); v[m].im = warp_sum(v[m].im); }
}

// the static integrals of one near pair by the whole warp (lanes over the
// rule's points, shuffle-reduced: every lane ends with the totals)
__device__ void fippi_warp(const DevNear& d, const double* Va, const double* Vb, const double* sgx, const double* sgw,
                           int n, int lane, Fippi& F) {
  fippi_zero(&F);
  if (d.ncv == 0) {
    double A[3], B[3], Ap[3], Bp[3], dV[3], a2;
    fippi_far_setup(Va, Vb, A, B, Ap, Bp, dV, &a2);
    for (int q = lane; q < n * n * n; q += 32) {
      const int i1 = q / (n * n), j = (q / n) % n, l = q % n;
      const double u = sgx[i1];
      fippi_far_acc(A, B, Ap, Bp, dV, a2, u, u * sgx[j], sgx[l], sgw[i1] * sgw[j] * sgw[l] * u, F);
    }
  } else {
    double Ea[9], Eb[9];
    touch_edges(Va, Vb, d.perm_a, d.perm_b, Ea, Eb);
    const int np = duffy_npts(d.ncv, n);
    DuffyPt pt;
    for (int q = lane; q < np; q += 32) {
      duffy_pt(d.ncv, q, sgx, sgw, n, pt);
      fippi_touch_acc(Ea, Eb, d.perm_a, d.perm_b, Va, pt, F);
    }
  }
  fippi_warp_sum(F);
}

__global__ void __launch_bounds__(FIPPI_THREADS) fippi_kernel(const DevNear* near, const int* list, int n,
                                                               const double* pv, Fippi* out) {
  __shared__ double sgx[N_FIP], sgw[N_FIP];
  if (threadIdx.x < N_FIP) { sgx[threadIdx.x] = c_gx12[threadIdx.x]; sgw[threadIdx.x] = c_gw12[threadIdx.x]; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (w >= n) return;  // whole warps
  const int i = list[w];
  const DevNear d = near[i];
  double Va[9], Vb[9];
#pragma unroll
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  Fippi F;
  fippi_zero(&F);
  if (d.ncv == 0) {
    double A[3], B[3], Ap[3], Bp[3], dV[3], a2;
    fippi_far_setup(Va, Vb, A, B, Ap, Bp, dV, &a2);
    for (int q = lane; q < N_FIP * N_FIP * N_FIP; q += 32) {
      const int i1 = q / (N_FIP * N_FIP), j = (q / N_FIP) % N_FIP, l = q % N_FIP;
      const double u = sgx[i1];
      fippi_far_acc(A, B, Ap, Bp, dV, a2, u, u * sgx[j], sgx[l], sgw[i1] * sgw[j] * sgw[l] * u, F);
    }
  } else {
    double Ea[9], Eb[9];
    touch_edges(Va, Vb, d.perm_a, d.perm_b, Ea, Eb);
    const int np = duffy_npts(d.ncv, N_FIP);
    DuffyPt pt;
    for (int q = lane; q < np; q += 32) {
      duffy_pt(d.ncv, q, sgx, sgw, N_FIP, pt);
      fippi_touch_acc(Ea, Eb, d.perm_a, d.perm_b, Va, pt, F);
    }
  }
  fippi_warp_sum(F);
  if (lane == 0) out[i] = F;
}

// ---------------------------------------------------------------------------
// per-frequency near pairs
// ---------------------------------------------------------------------------
__device__ void store_near(double* dst, int ja, int jb, cx<double> kk, cx<double> kn, cx<double> nn) {
  double* o = dst + 6 * (3 * ja + jb);
  o[0] += kk.re; o[1] += kk.im; o[2] += kn.re; o[3] += kn.im; o[4] += nn.re; o[5] += nn.im;
}

// one warp per common-triangle pair: the 6*NT_SELF outer points are split
// over the lanes and the moments reduced with shuffles
__global__ void __launch_bounds__(128) self_kernel(const DevNear* near, const int* list, int n, const double* pv,
                                                   RegionArgs ra, double* nearval) {
  // the 1-D rule in shared memory: the lanes read different nodes at once
  __shared__ double sgx[NT_SELF], sgw[NT_SELF];
  if (threadIdx.x < NT_SELF) { sgx[threadIdx.x] = c_gx16[threadIdx.x]; sgw[threadIdx.x] = c_gw16[threadIdx.x]; }
  __syncthreads();
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;  // whole warps exit together
  int i = list[warp];
  DevNear d = near[i];
  double V[9];
  for (int c = 0; c < 9; c++) V[c] = pv[9 * (size_t)d.pa + c];
  double* dst = nearval + 54 * (size_t)i;
  // lane q < 9 accumulates combination q = 3 ja + jb: KK (re, im), KN (zero), NN (re, im)
  double acc0 = 0.0, acc1 = 0.0, acc4 = 0.0, acc5 = 0.0;
  for (int r = 0; r < ra.nreg; r++) {
    cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    cx<double> MG[9], MP[9];
    self_moments(V, k, sgx, sgw, NT_SELF, MG, lane, 32);
    for (int m = 0; m < 9; m++) {
      for (int o = 16; o > 0; o >>= 1) {
        MG[m].re += __shfl_xor_sync(0xffffffff, MG[m].re, o);
        MG[m].im += __shfl_xor_sync(0xffffffff, MG[m].im, o);
      }
      MP[m] = mk(0.0, 0.0);
    }
    cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
    if (lane < 9) {
      int ja = lane / 3, jb = lane % 3;
      double c[9], dd[9];
      combo_coeffs(V, V, ja, jb, c, dd);
      cx<double> H0, H1;
      combine(MG, MP, c, dd, m4ok2, &H0, &H1);
      cx<double> v0 = ra.pf1[r] * H0, v2 = ra.pf3[r] * H0;
      acc0 += v0.re; acc1 += v0.im;
      acc4 += v2.re; acc5 += v2.im;
    }
  }
  if (lane < 9) {
    double* o = dst + 6 * lane;
    o[0] = acc0; o[1] = acc1; o[2] = 0.0; o[3] = 0.0; o[4] = acc4; o[5] = acc5;
  }
}

__global__ void near_kernel(const DevNear* near, const int* list, int n, const double* pv, const Fippi* fippi,
                            RegionArgs ra, double* nearval, int* status) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int i = list[t];
  DevNear d = near[i];
  double Va[9], Vb[9];
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  double* dst = nearval + 54 * (size_t)i;
  for (int c = 0; c < 54; c++) dst[c] = 0.0;
  const Fippi& F = fippi[i];  // read where used: keeps 33 doubles out of registers
  for (int r = 0; r < ra.nreg; r++) {
    cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    // short-wavelength test of PanelPanelInteractions.cc:416-418
    cx<double> kr = mk(k.re * d.rmax, k.im * d.rmax);
    bool sw = hypot(kr.re, kr.im) > M_PI;
    cx<double> MG[9], MP[9];
    bool desing = false;
    if (!sw) {
      pair_moments<double, 1>(g, k, c_lo64, 6, MG, MP);
      add_taylor_terms(F, k, MG, MP);
      desing = true;
    } else if (d.ncv == 0) {
      pair_moments<double, 0>(g, k, c_ho, HO_N * HO_N, MG, MP);
    } else {
      // touching pair in the short-wavelength regime: td_touch_kernel adds
      // this region's full-kernel Taylor-Duffy values after this kernel
      continue;
    }
    cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
    VecMoments<double> vm;
    vec_moments(g, MG, MP, &vm);
    for (int ja = 0; ja < 3; ja++)
      for (int jb = 0; jb < 3; jb++) {
        cx<double> H0, H1;
        vec_combine(g, vm, ja, jb, m4ok2, &H0, &H1);
        if (desing) H1 = H1 + mk(-0.079577471545947667884 * htimes_rm3(F, Va, Vb, ja, jb), 0.0);
        store_near(dst, ja, jb, ra.pf1[r] * H0, ra.pfc[r] * H1, ra.pf3[r] * H0);
      }
  }
}

// One warp per touching pair (ncv = 1, 2) in the short-wavelength regime
// (|k rmax| > pi, PanelPanelInteractions.cc:416-418): the Duffy points are
// split over the lanes, the 9 G moments and 10 H1 moments reduced with
// shuffles, and lanes 0..8 add the nine (Qa,Qb) combinations.
constexpr int N_TD = 12;  // Gauss points per Duffy dimension
__global__ void __launch_bounds__(128) td_touch_kernel(const DevNear* near, const int* list, int n, const double* pv,
                                                       RegionArgs ra, double* nearval) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;  // whole warps exit together
  const int i = list[warp];
  const DevNear d = near[i];
  if (d.ncv < 1 || d.ncv > 2) return;
  double Va[9], Vb[9];
  for (int c = 0; c < 9; c++) { Va[c] = pv[9 * (size_t)d.pa + c]; Vb[c] = pv[9 * (size_t)d.pb + c]; }
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  double* dst = nearval + 54 * (size_t)i;
  for (int r = 0; r < ra.nreg; r++) {
    const cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    if (!(hypot(k.re * d.rmax, k.im * d.rmax) > M_PI)) continue;  // near_kernel's desingularised branch
    cx<double> MG[9], T[10];
    td_touch(d.ncv, Va, Vb, d.perm_a, d.perm_b, k, c_gx12, c_gw12, N_TD, lane, 32, MG, T);
    for (int m = 0; m < 9; m++)
      for (int o = 16; o > 0; o >>= 1) {
        MG[m].re += __shfl_xor_sync(0xffffffff, MG[m].re, o);
        MG[m].im += __shfl_xor_sync(0xffffffff, MG[m].im, o);
      }
    for (int m = 0; m < 10; m++)
      for (int o = 16; o > 0; o >>= 1) {
        T[m].re += __shfl_xor_sync(0xffffffff, T[m].re, o);
        T[m].im += __shfl_xor_sync(0xffffffff, T[m].im, o);
      }
    if (lane < 9) {
      const int ja = lane / 3, jb = lane % 3;
      cx<double> MP[9];
      for (int m = 0; m < 9; m++) MP[m] = mk(0.0, 0.0);
      VecMoments<double> vm;
      vec_moments(g, MG, MP, &vm);
      cx<double> H0, H1unused;
      vec_combine(g, vm, ja, jb, cdiv(mk(-4.0, 0.0), k * k), &H0, &H1unused);
      const cx<double> H1 = td_h1(Va, Vb, T, ja, jb);
      store_near(dst, ja, jb, ra.pf1[r] * H0, ra.pfc[r] * H1, ra.pf3[r] * H0);
    }
  }
}

// ---------------------------------------------------------------------------
// far-field tile kernel
// ---------------------------------------------------------------------------
struct TileArgs {
  const DevEdgeBlock* rows;
  const DevEdgeBlock* cols;
  const int2* tiles;
  const double* pv;
  const double* pc;
  const double* elen_a;
  const double* elen_b;
  const int* nptr;
  const int* ncol;
  const int* nidx;
  const double* nearval;
  int row_panel_offset;
  int bpe_a, bpe_b;
  int row_off, col_off;    // where entry (row edge, col edge) of the block goes
  int mrow_off, mcol_off;  // where its mirror (col edge, row edge) goes
  int passes;              // bit 0: write the block, bit 1: write the mirror
  int sym;
  void* out;
  long long ld;
};

// relative distance with the reference's operation order and no FMA
// contraction (AssessPanelPair.cc:160-166)
__device__ __forceinline__ bool is_far(const double* ca, const double* cb, double ra, double rb) {
  double rmax = fmax(ra, rb);
  double dc = __dsub_rn(ca[0], cb[0]);
  double r2 = __dmul_rn(dc, dc);
  dc = __dsub_rn(ca[1], cb[1]);
  r2 = __dadd_rn(r2, __dmul_rn(dc, dc));
  dc = __dsub_rn(ca[2], cb[2]);
  r2 = __dadd_rn(r2, __dmul_rn(dc, dc));
  return __ddiv_rn(__dsqrt_rn(r2), rmax) > 4.0;
}

// rRel > 4 decides the 6x6 rule; an FP32 estimate settles all but the pairs
// within 1e-4 of the threshold, which take the exact FP64 test
__device__ __forceinline__ bool tile_pair_far(const float* ca, const float* cb, const double* da, const double* db) {
  const float dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
  const float d2f = dx * dx + dy * dy + dz * dz, rmf = fmaxf(ca[3], cb[3]);
  if (d2f > 16.0008f * rmf * rmf) return true;
  if (d2f < 15.9992f * rmf * rmf) return false;
  return is_far(da, db, da[3], db[3]);
}

// index of the near pair (global panels gpa, gpb) in the block's near list,
// times 2, plus 1 when it is stored transposed; -1 if absent
__device__ __forceinline__ int near_hit(const TileArgs& a, int gpa, int gpb) {
  const int row = gpa - a.row_panel_offset;
  for (int e = a.nptr[row]; e < a.nptr[row + 1]; e++)
    if (a.ncol[e] == gpb) return a.nidx[e];
  return -1;
}

// tile entry q of a pass: pass 0 walks column-major (coalesced stores into
// the block), pass 1 row-major (coalesced stores into its mirror).  A
// diagonal tile of a symmetric block writes its upper triangle and mirrors
// it, so the matrix is exactly symmetric (AssembleBEMMatrix.cc:753-758).
__device__ __forceinline__ bool tile_entry(int pass, int q, int NR, int NCc, bool diag, int* i, int* j) {
  if (pass == 0) { *i = q % NR; *j = q / NR; } else { *j = q % NCc; *i = q / NCc; }
  return !(diag && (pass == 0 ? *i > *j : *i >= *j));
}

// write entry (row edge ea, column edge eb) of the block -- pass 0 -- or its
// mirror -- pass 1 -- with the (dx, dy) sub-entries of dielectric basis
// pairs: e00 = EE, e01 = e10 = EH/HE, e11 = HH
template <typename C>
__device__ __forceinline__ void store_entry(const TileArgs& a, C* out, int pass, int ea, int eb, C e00, C eoff, C e11) {
  const long long ld = a.ld;
  const long long X = (pass == 0 ? a.row_off : a.mcol_off) + (long long)a.bpe_a * ea;
  const long long Y = (pass == 0 ? a.col_off : a.mrow_off) + (long long)a.bpe_b * eb;
  if (a.bpe_a == 1 && a.bpe_b == 1) {
    if (pass == 0) out[X + Y * ld] = e00; else out[Y + X * ld] = e00;
  } else if (a.bpe_a == 1) {
    if (pass == 0) { out[X + Y * ld] = e00; out[X + (Y + 1) * ld] = eoff; }
    else { out[Y + X * ld] = e00; out[(Y + 1) + X * ld] = eoff; }
  } else if (a.bpe_b == 1) {
    if (pass == 0) { out[X + Y * ld] = e00; out[(X + 1) + Y * ld] = eoff; }
    else { out[Y + X * ld] = e00; out[Y + (X + 1) * ld] = eoff; }
  } else {
    if (pass == 0) {
      out[X + Y * ld] = e00; out[X + 1 + Y * ld] = eoff;
      out[X + (Y + 1) * ld] = eoff; out[X + 1 + (Y + 1) * ld] = e11;
    } else {
      out[Y + X * ld] = e00; out[Y + 1 + X * ld] = eoff;
      out[Y + (X + 1) * ld] = eoff; out[Y + 1 + (X + 1) * ld] = e11;
    }
  }
}

// FP64 far field: one CTA per tile of TE x TE edge pairs (upper triangle of
// symmetric blocks).  The CTA stages its panels in shared memory, computes
// the moments of every panel pair the tile touches once, forms the needed
// (Qa,Qb) combinations and writes each into a per-(edge pair, P/M side) slot;
// every slot has one writer, so the four contributions of an edge pair are
// summed in a fixed order (deterministic, no atomics).
template <int NC>
__global__ void __launch_bounds__(256) tile_kernel(TileArgs a, RegionArgs ra) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<double>* slots = reinterpret_cast<cx<double>*>(smem_raw);  // [TE][TE][4][NC]
  __shared__ double s_pv[2][PMAX][9];
  __shared__ double s_pc[2][PMAX][4];
  __shared__ int8_t s_hl[2][3 * PMAX], s_hs[2][3 * PMAX];
  __shared__ int s_gp[2][PMAX];
  __shared__ float s_cf[2][PMAX][4];  // FP32 centroid and radius (pre-check of rRel)

  const int2 tile = a.tiles[blockIdx.x];
  const DevEdgeBlock* RB = a.rows + tile.x;
  const DevEdgeBlock* CB = a.cols + tile.y;
  const int PR = RB->np, PC = CB->np, NR = RB->ne, NCc = CB->ne;
  for (int q = threadIdx.x; q < PR * 9; q += blockDim.x) s_pv[0][q / 9][q % 9] = a.pv[9 * (size_t)RB->panels[q / 9] + q % 9];
  for (int q = threadIdx.x; q < PC * 9; q += blockDim.x) s_pv[1][q / 9][q % 9] = a.pv[9 * (size_t)CB->panels[q / 9] + q % 9];
  for (int q = threadIdx.x; q < PR * 4; q += blockDim.x) s_pc[0][q / 4][q % 4] = a.pc[4 * (size_t)RB->panels[q / 4] + q % 4];
  for (int q = threadIdx.x; q < PC * 4; q += blockDim.x) s_pc[1][q / 4][q % 4] = a.pc[4 * (size_t)CB->panels[q / 4] + q % 4];
  for (int q = threadIdx.x; q < 3 * PR; q += blockDim.x) { s_hl[0][q] = RB->hl[q]; s_hs[0][q] = RB->hs[q]; }
  for (int q = threadIdx.x; q < 3 * PC; q += blockDim.x) { s_hl[1][q] = CB->hl[q]; s_hs[1][q] = CB->hs[q]; }
  for (int q = threadIdx.x; q < PR; q += blockDim.x) s_gp[0][q] = RB->panels[q];
  for (int q = threadIdx.x; q < PC; q += blockDim.x) s_gp[1][q] = CB->panels[q];
  __syncthreads();
  for (int q = threadIdx.x; q < 2 * PMAX; q += blockDim.x) {
    const int side = q / PMAX, p = q % PMAX;
    if (p < (side ? PC : PR))
      for (int c = 0; c < 4; c++) s_cf[side][p][c] = (float)s_pc[side][p][c];
  }
  __syncthreads();

  for (int q = threadIdx.x; q < PR * PC; q += blockDim.x) {
    const int ia = q / PC, ib = q - ia * PC;
    const double* Va = s_pv[0][ia];
    const double* Vb = s_pv[1][ib];
    int la[3], lb[3], sa[3], sb[3];
    for (int j = 0; j < 3; j++) {
      la[j] = s_hl[0][3 * ia + j]; sa[j] = s_hs[0][3 * ia + j];
      lb[j] = s_hl[1][3 * ib + j]; sb[j] = s_hs[1][3 * ib + j];
    }
    if (tile_pair_far(s_cf[0][ia], s_cf[1][ib], s_pc[0][ia], s_pc[1][ib])) {
      PairGeom<double> g;
      for (int c = 0; c < 3; c++) {
        g.D0[c] = Va[c] - Vb[c];
        g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
        g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
      }
      bool first = true;
      for (int r = 0; r < ra.nreg; r++) {
        cx<double> k = ra.k[r];
        if (k.re == 0.0 && k.im == 0.0) continue;
        cx<double> MG[9], MP[9];
        pair_moments<double, 0>(g, k, c_lo64, 6, MG, MP);
        const cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
        for (int ja = 0; ja < 3; ja++) {
          if (la[ja] < 0) continue;
          for (int jb = 0; jb < 3; jb++) {
            if (lb[jb] < 0) continue;
            double c[9], d[9];
            combo_coeffs(Va, Vb, ja, jb, c, d);
            cx<double> H0, H1;
            combine(MG, MP, c, d, m4ok2, &H0, &H1);
            cx<double>* sl = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
            const cx<double> v0 = ra.pf1[r] * H0;
            if (first) sl[0] = v0; else sl[0] = sl[0] + v0;
            if (NC > 1) { const cx<double> v1 = ra.pfc[r] * H1; if (first) sl[1] = v1; else sl[1] = sl[1] + v1; }
            if (NC > 2) { const cx<double> v2 = ra.pf3[r] * H0; if (first) sl[2] = v2; else sl[2] = sl[2] + v2; }
          }
        }
        first = false;
      }
      if (first) {  // every common region has k = 0: zero contribution
        for (int ja = 0; ja < 3; ja++)
          for (int jb = 0; jb < 3; jb++)
            if (la[ja] >= 0 && lb[jb] >= 0) {
              cx<double>* sl = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
              for (int c = 0; c < NC; c++) sl[c] = mk(0.0, 0.0);
            }
      }
    } else {
      // near pair: values precomputed in FP64 by self_kernel / near_kernel
      const int hit = near_hit(a, s_gp[0][ia], s_gp[1][ib]);
      if (hit < 0) continue;  // cannot happen: every rRel<=4 pair is listed
      const double* nv = a.nearval + 54 * (size_t)(hit >> 1);
      const bool tr = hit & 1;
      for (int ja = 0; ja < 3; ja++) {
        if (la[ja] < 0) continue;
        for (int jb = 0; jb < 3; jb++) {
          if (lb[jb] < 0) continue;
          const double* v = nv + 6 * (tr ? (3 * jb + ja) : (3 * ja + jb));
          cx<double>* sl = slots + ((size_t)(la[ja] * TE + lb[jb]) * 4 + sa[ja] * 2 + sb[jb]) * NC;
          sl[0] = mk(v[0], v[1]);
          if (NC > 1) sl[1] = mk(v[2], v[3]);
          if (NC > 2) sl[2] = mk(v[4], v[5]);
        }
      }
    }
  }
  __syncthreads();

  // entries: sum of the four P/M contributions times La Lb
  cx<double>* out = reinterpret_cast<cx<double>*>(a.out);
  const bool diag = a.sym && tile.x == tile.y;
  for (int pass = 0; pass < 2; pass++) {
    if (!(a.passes & (1 << pass))) continue;
    for (int q = threadIdx.x; q < NR * NCc; q += blockDim.x) {
      int i, j;
      if (!tile_entry(pass, q, NR, NCc, diag, &i, &j)) continue;
      const cx<double>* sl = slots + (size_t)(i * TE + j) * 4 * NC;
      const double L = a.elen_a[RB->e0 + i] * a.elen_b[CB->e0 + j];
      cx<double> v[3];
      for (int c = 0; c < NC; c++) v[c] = L * ((sl[c] - sl[NC + c]) - (sl[2 * NC + c] - sl[3 * NC + c]));
      store_entry(a, out, pass, RB->e0 + i, CB->e0 + j, v[0], NC > 1 ? v[1] : v[0], NC > 2 ? v[2] : v[0]);
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed-precision far field, on the FP32 pipes in float-float arithmetic
// (ffmath.cuh), in two passes per column stripe of a block:
//  1. ppair_kernel: every far panel pair (row panel, stripe column panel)
//     once -- moments for each common region, then the slot values of all 9
//     (Qa, Qb) choices, EE/HH channels as float-float and the EH channel in
//     FP32 -- into a scratch buffer; near pairs get a NaN marker.
//  2. stamp_kernel: per edge tile, each entry sums its four (P/M, P/M)
//     values (from the buffer, or from the FP64 near table) in float-float,
//     applies La Lb, rounds to complex64 once, and is written with its mirror.
// Computing each panel pair once (the tile kernel recomputes a panel pair in
// every tile that touches it, ~2.4x over on an icosphere) and without the
// 190 KB of float-float slots per CTA is what makes the float-float form
// affordable.
// ---------------------------------------------------------------------------
constexpr int NODE_STRIDE = 37;  // floats per panel in shared memory: 6 nodes x (3 hi + 3 lo), + 1 (bank spread)
constexpr int GEO_STRIDE = 19;   // floats per panel in shared memory: V0 - O, A, B as float-float, + 1

template <int NC> constexpr int ppair_fields() { return NC == 1 ? 4 : (NC == 2 ? 6 : 10); }

struct PPairArgs {
  const float* node;  // per global panel: 36 floats (float-float rule nodes)
  const float* geo;   // per global panel: 18 floats (float-float V0 - O, A, B)
  const double* pc;   // per global panel: centroid, radius
  const int* cpan;    // the stripe's column panels (surface-local)
  int offa, offb;     // global index of the first panel of each surface
  int nrow, ncp;
  float* out;         // [NF][9][ncp][nrow]
};

// pass 1: block (32, PP_COLS) = 32 row panels x PP_COLS column panels, one
// pair per thread; 168 registers let 12 warps share an SM
constexpr int PP_COLS = 12, PP_SLOTS = 32 + PP_COLS, PP_THREADS = 32 * PP_COLS;

template <int NC>
__global__ void __launch_bounds__(PP_THREADS, 1) ppair_kernel(PPairArgs p, RegionArgs ra) {
  constexpr int NF = ppair_fields<NC>();
  __shared__ float s_node[PP_SLOTS][NODE_STRIDE];
  __shared__ float s_geo[PP_SLOTS][GEO_STRIDE];
  __shared__ double s_pcd[PP_SLOTS][4];
  __shared__ float s_cf[PP_SLOTS][4];
  __shared__ SinCosTab s_tab;
  __shared__ FFRule s_rule;
  __shared__ cff s_k[2], s_m4[2], s_p1[2], s_p3[2];  // s_k[r] = (Re k, Im k) as float-float
  __shared__ cx<float> s_pcf[2];
  __shared__ int s_live[2];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * PP_COLS;
  // the CTA's 32 row and PP_COLS column panels (global index, -1 past the end)
  auto panel_of = [&](int sl) -> int {
    if (sl < 32) return r0 + sl < p.nrow ? p.offa + r0 + sl : -1;
    return c0 + sl - 32 < p.ncp ? p.offb + p.cpan[c0 + sl - 32] : -1;
  };
  for (int q = tid; q < PP_SLOTS * 36; q += PP_THREADS) {
    const int sl = q / 36, f = q - sl * 36, gp = panel_of(sl);
    if (gp >= 0) s_node[sl][f] = p.node[36 * (size_t)gp + f];
  }
  for (int q = tid; q < PP_SLOTS * 18; q += PP_THREADS) {
    const int sl = q / 18, f = q - sl * 18, gp = panel_of(sl);
    if (gp >= 0) s_geo[sl][f] = p.geo[18 * (size_t)gp + f];
  }
  for (int q = tid; q < PP_SLOTS * 4; q += PP_THREADS) {
    const int sl = q / 4, f = q - sl * 4, gp = panel_of(sl);
    if (gp >= 0) { s_pcd[sl][f] = p.pc[4 * (size_t)gp + f]; s_cf[sl][f] = (float)p.pc[4 * (size_t)gp + f]; }
  }
  for (int q = tid; q < (int)(sizeof(SinCosTab) / 4); q += PP_THREADS)
    reinterpret_cast<float*>(&s_tab)[q] = reinterpret_cast<const float*>(&c_sctab)[q];
  for (int q = tid; q < (int)(sizeof(FFRule) / 4); q += PP_THREADS)
    reinterpret_cast<float*>(&s_rule)[q] = reinterpret_cast<const float*>(&c_ffrule)[q];
  if (tid < 2) {
    // region constants, formed once per CTA in FP64
    const int r = tid;
    const cx<double> kd = r < ra.nreg ? ra.k[r] : mk(0.0, 0.0);
    const bool live = !(kd.re == 0.0 && kd.im == 0.0);
    s_live[r] = live;
    s_k[r] = cff_of(kd);
    s_m4[r] = live ? cff_of(cdiv(mk(-4.0, 0.0), kd * kd)) : cff_zero();
    s_p1[r] = live ? cff_of(ra.pf1[r]) : cff_zero();
    s_p3[r] = live ? cff_of(ra.pf3[r]) : cff_zero();
    s_pcf[r] = live ? mk((float)ra.pfc[r].re, (float)ra.pfc[r].im) : mk(0.0f, 0.0f);
  }
  __syncthreads();

  const int pa = r0 + threadIdx.x, cl = c0 + threadIdx.y;
  if (pa >= p.nrow || cl >= p.ncp) return;
  const int ia = threadIdx.x, ib = 32 + threadIdx.y;
  const size_t cs = (size_t)p.ncp * p.nrow;  // stride of one (field, combination) plane
  float* out = p.out + (size_t)cl * p.nrow + pa;
  if (!tile_pair_far(s_cf[ia], s_cf[ib], s_pcd[ia], s_pcd[ib])) {
    const float marker = __int_as_float(0x7fc00000);  // quiet NaN: a near pair
    for (int c = 0; c < 9; c++) out[c * cs] = marker;
    return;
  }
  FFGeom g;
  for (int c = 0; c < 3; c++) {
    g.Aa[c] = ffv(s_geo[ia][6 + c], s_geo[ia][9 + c]); g.Ba[c] = ffv(s_geo[ia][12 + c], s_geo[ia][15 + c]);
    g.Ab[c] = ffv(s_geo[ib][6 + c], s_geo[ib][9 + c]); g.Bb[c] = ffv(s_geo[ib][12 + c], s_geo[ib][15 + c]);
    g.D0[c] = ff_sub(ffv(s_geo[ia][c], s_geo[ia][3 + c]), ffv(s_geo[ib][c], s_geo[ib][3 + c]));
  }
  ff D[2][2];
  h0_dots(g, D);
  H1Pre p1;
  if (NC > 1) h1_prepare(g, &p1);
  constexpr int R2 = NC == 1 ? 1 : 2;
  for (int r = 0; r < R2; r++) {
    const bool live = s_live[r];
    if (r > 0 && !live) break;
    cff MP[9];
    H0Pre p0;
    if (live) {
      cff MG[9];
      pair_moments_ff<6>(s_node[ia], s_node[ib], s_k[r].re, s_k[r].im, &s_rule, &s_tab, MG, MP);
      h0_prepare(D, MG, &p0);
    }
#pragma unroll 1
    for (int c = 0; c < 9; c++) {
      const int ja = c / 3, jb = c - 3 * ja;
      cff v0 = cff_zero(), v2 = cff_zero();
      cx<float> v1 = mk(0.0f, 0.0f);
      if (live) {
        const cff H0 = h0_combo(p0, ja, jb, s_m4[r]);
        v0 = cff_mul(s_p1[r], H0);
        if (NC > 2) v2 = cff_mul(s_p3[r], H0);
        if (NC > 1) {
          const cff H1 = h1_combo(p1, ja, jb, MP);
          v1 = s_pcf[r] * mk(H1.re.hi + H1.re.lo, H1.im.hi + H1.im.lo);
        }
      }
      float* o = out + c * cs;
      const size_t fs = 9 * cs;  // stride of one field
      if (r > 0) {
        // the second region adds to the first (same thread: no ordering issue)
        v0 = cff_add(v0, cffv(ffv(o[0], o[fs]), ffv(o[2 * fs], o[3 * fs])));
        if (NC > 1) v1 = v1 + mk(o[4 * fs], o[5 * fs]);
        if (NC > 2) v2 = cff_add(v2, cffv(ffv(o[6 * fs], o[7 * fs]), ffv(o[8 * fs], o[9 * fs])));
      }
      o[0] = v0.re.hi; o[fs] = v0.re.lo; o[2 * fs] = v0.im.hi; o[3 * fs] = v0.im.lo;
      if (NC > 1) { o[4 * fs] = v1.re; o[5 * fs] = v1.im; }
      if (NC > 2) { o[6 * fs] = v2.re.hi; o[7 * fs] = v2.re.lo; o[8 * fs] = v2.im.hi; o[9 * fs] = v2.im.lo; }
    }
  }
  (void)NF;
}

struct StampArgs {
  TileArgs ta;            // output placement, near table, edge blocks
  const int2* tiles;      // the stripe's tiles
  const int4* edge_a;     // per row edge: P panel, its Q index, M panel, its Q index (surface-local; -1: none)
  const int4* edge_b;     // per column edge, likewise
  const int2* ecol;       // per column edge: stripe-local index of its P, M panel
  int offb;               // global index of the first column-surface panel
  const float* ppv;       // pass-1 values [NF][9][ncp][nrow]
  int nrow, ncp;
};

// pass 2: one CTA per edge tile; the entries are formed once into shared
// memory, then written column-major (block) and row-major (mirror) so both
// stores are coalesced
template <int NC>
__global__ void __launch_bounds__(256) stamp_kernel(StampArgs sp) {
  __shared__ cx<float> s_val[TE * TE * NC];
  const TileArgs& a = sp.ta;
  const int2 tile = sp.tiles[blockIdx.x];
  const DevEdgeBlock* RB = a.rows + tile.x;
  const DevEdgeBlock* CB = a.cols + tile.y;
  const int NR = RB->ne, NCc = CB->ne;
  const bool diag = a.sym && tile.x == tile.y;
  const size_t cs = (size_t)sp.ncp * sp.nrow, fs = 9 * cs;
  for (int q = threadIdx.x; q < NR * NCc; q += blockDim.x) {
    const int i = q % NR, j = q / NR;
    if (diag && i > j) continue;
    const int ea = RB->e0 + i, eb = CB->e0 + j;
    const int4 A = sp.edge_a[ea], B = sp.edge_b[eb];
    const int2 C = sp.ecol[eb];
    cff s0 = cff_zero(), s2 = cff_zero();
    cx<float> s1 = mk(0.0f, 0.0f);
    for (int u = 0; u < 2; u++) {
      const int pa = u ? A.z : A.x, ja = u ? A.w : A.y;
      if (pa < 0) continue;
      for (int w = 0; w < 2; w++) {
        const int pb = w ? B.z : B.x, jb = w ? B.w : B.y, cl = w ? C.y : C.x;
        if (pb < 0) continue;
        const float* src = sp.ppv + (size_t)(3 * ja + jb) * cs + (size_t)cl * sp.nrow + pa;
        cff v0, v2 = cff_zero();
        cx<float> v1 = mk(0.0f, 0.0f);
        const float f0 = src[0];
        if (!isnan(f0)) {
          v0 = cffv(ffv(f0, src[fs]), ffv(src[2 * fs], src[3 * fs]));
          if (NC > 1) v1 = mk(src[4 * fs], src[5 * fs]);
          if (NC > 2) v2 = cffv(ffv(src[6 * fs], src[7 * fs]), ffv(src[8 * fs], src[9 * fs]));
        } else {
          // near pair: FP64 values of near_kernel / self_kernel
          const int hit = near_hit(a, a.row_panel_offset + pa, sp.offb + pb);
          if (hit < 0) continue;  // cannot happen: every rRel<=4 pair is listed
          const double* v = a.nearval + 54 * (size_t)(hit >> 1) + 6 * ((hit & 1) ? (3 * jb + ja) : (3 * ja + jb));
          v0 = cff_of(mk(v[0], v[1]));
          if (NC > 1) v1 = mk((float)v[2], (float)v[3]);
          if (NC > 2) v2 = cff_of(mk(v[4], v[5]));
        }
        if (u == w) {
          s0 = cff_add(s0, v0); s1 = s1 + v1; s2 = cff_add(s2, v2);
        } else {
          s0 = cff_sub(s0, v0); s1 = s1 - v1; s2 = cff_sub(s2, v2);
        }
      }
    }
    // La Lb in FP64, then float-float: an FP32 product would scale every row
    // and column of an edge by its own rounding, which the right-hand side
    // and the power integrals do not share
    const ff L = ff_of(a.elen_a[ea] * a.elen_b[eb]);
    cx<float>* o = s_val + (size_t)(i * TE + j) * NC;
    const cff y0 = cff_mul_ff(s0, L);
    o[0] = mk(y0.re.hi + y0.re.lo, y0.im.hi + y0.im.lo);
    if (NC > 1) o[1] = mk(fmaf(L.hi, s1.re, L.lo * s1.re), fmaf(L.hi, s1.im, L.lo * s1.im));
    if (NC > 2) {
      const cff y2 = cff_mul_ff(s2, L);
      o[2] = mk(y2.re.hi + y2.re.lo, y2.im.hi + y2.im.lo);
    }
  }
  __syncthreads();
  cx<float>* out = reinterpret_cast<cx<float>*>(a.out);
  for (int pass = 0; pass < 2; pass++) {
    if (!(a.passes & (1 << pass))) continue;
    for (int q = threadIdx.x; q < NR * NCc; q += blockDim.x) {
      int i, j;
      if (!tile_entry(pass, q, NR, NCc, diag, &i, &j)) continue;
      const cx<float>* v = s_val + (size_t)(i * TE + j) * NC;
      store_entry(a, out, pass, RB->e0 + i, CB->e0 + j, v[0], NC > 1 ? v[1] : v[0], NC > 2 ? v[2] : v[0]);
    }
  }
}

static inline cx<double> cxd(double r, double i) { return mk(r, i); }

template <int NC>
static cudaError_t launch_tiles64(const TileArgs& ta, const RegionArgs& ra, int ntiles, cudaStream_t s) {
  const size_t smem = (size_t)TE * TE * 4 * NC * sizeof(cx<double>);
  cudaError_t e = allow_max_smem(tile_kernel<NC>);
  if (e != cudaSuccess) return e;
  tile_kernel<NC><<<ntiles, 256, smem, s>>>(ta, ra);
  return cudaGetLastError();
}

// the two passes of the mixed far field over a block's column stripes
template <int NC>
static cudaError_t far_mixed(Geometry* g, const Block& b, DevBlock* db, const TileArgs& ta, const RegionArgs& ra,
                             cudaStream_t s) {
  const size_t need = b.max_stripe_pairs * 9 * ppair_fields<NC>() * sizeof(float);
  cudaError_t e = cudaSuccess;
  if (need > g->ppv_bytes) {
    // grow the scratch (kept on the geometry; the old one may still be read
    // by earlier launches, so wait for the device before freeing it)
    if (g->ppv) {
      e = cudaDeviceSynchronize();
      cudaFree(g->ppv);
    }
    g->ppv = nullptr;
    g->ppv_bytes = 0;
    if (e == cudaSuccess) e = cudaMalloc(&g->ppv, need);
    if (e != cudaSuccess) return e;
    g->ppv_bytes = need;
  }
  for (const DevBlock::DevStripe& st : db->stripes) {
    if (st.ntiles == 0 || st.ncp == 0) continue;
    PPairArgs pp;
    pp.node = g->d_ffnode; pp.geo = g->d_ffgeo; pp.pc = g->d_pc; pp.cpan = st.cpan;
    pp.offa = g->S[b.sa].panel_offset; pp.offb = g->S[b.sb].panel_offset;
    pp.nrow = st.nrow; pp.ncp = st.ncp; pp.out = (float*)g->ppv;
    ppair_kernel<NC><<<dim3((st.nrow + 31) / 32, (st.ncp + PP_COLS - 1) / PP_COLS), dim3(32, PP_COLS), 0, s>>>(pp, ra);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    StampArgs sp;
    sp.ta = ta; sp.tiles = st.tiles; sp.edge_a = db->edge_a; sp.edge_b = db->edge_b; sp.ecol = db->ecol;
    sp.offb = pp.offb; sp.ppv = pp.out; sp.nrow = st.nrow; sp.ncp = st.ncp;
    stamp_kernel<NC><<<st.ntiles, 256, 0, s>>>(sp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    stats_launch(ST_FAR, 2);
  }
  return cudaSuccess;
}

// The static table of every near pair.  With records in the process-wide
// cache (gbem_cache_preload), the pairs found there are converted on the host
// and uploaded, and the kernel computes only the others.
gbem_status compute_fippi(Geometry* g, cudaStream_t s) {
  const bool cached = cache_active();
  for (size_t bi = 0; bi < g->blocks.size(); bi++) {
    DevBlock* db = g->dblocks[bi];
    if (db->nother == 0) continue;
    StatTimer t(ST_NEAR, s);
    const int* list = db->other_list;
    int n = db->nother;
    int* dmiss = nullptr;
    if (cached) {
      std::vector<Fippi> table;
      std::vector<int> miss;
      cache_lookup(g, g->blocks[bi], table, miss);
      cudaError_t e = cudaMemcpyAsync(db->fippi, table.data(), sizeof(Fippi) * table.size(), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess && !miss.empty()) e = cudaMallocAsync((void**)&dmiss, sizeof(int) * miss.size(), s);
      if (e == cudaSuccess && !miss.empty())
        e = cudaMemcpyAsync(dmiss, miss.data(), sizeof(int) * miss.size(), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host vectors go out of scope
      if (e != cudaSuccess) return cuda_status(e, "cached near table");
      list = dmiss;
      n = (int)miss.size();
    }
    if (n > 0) {
      fippi_kernel<<<(unsigned)(((long long)n * 32 + FIPPI_THREADS - 1) / FIPPI_THREADS), FIPPI_THREADS, 0, s>>>(
          db->near, list, n, g->d_pv, db->fippi);
      stats_launch(ST_NEAR);
    }
    cudaError_t e = cudaGetLastError();
    if (dmiss) cudaFreeAsync(dmiss, s);
    if (e != cudaSuccess) return cuda_status(e, "fippi_kernel");
  }
  g->fippi_ready = true;
  return GBEM_OK;
}

gbem_status download_fippi(Geometry* g, size_t bi, std::vector<Fippi>& table) {
  const DevBlock* db = g->dblocks[bi];
  table.assign((size_t)db->nnear, Fippi());
  if (!db->nnear) return GBEM_OK;
  cudaError_t e = cudaSetDevice(g->device);
  if (e == cudaSuccess) e = cudaMemcpy(table.data(), db->fippi, sizeof(Fippi) * table.size(), cudaMemcpyDeviceToHost);
  return cuda_status(e, "download near table");
}

// per-region wavenumbers and PMCHWT/EFIE prefactors of a surface block
// (SurfaceSurfaceInteractions.cc:165-176), signs folded in
static RegionArgs region_args(const Block& b, double wr, double wi, const double* eps, const double* mu) {
  RegionArgs ra;
  memset(&ra, 0, sizeof ra);
  ra.nreg = b.nreg;
  const cx<double> omega = cxd(wr, wi);
  for (int r = 0; r < b.nreg; r++) {
    int R = b.reg[r];
    cx<double> ep = cxd(eps[2 * R], eps[2 * R + 1]), m = cxd(mu[2 * R], mu[2 * R + 1]);
    // k = csqrt2(eps mu) omega, the root with Im >= 0 (libhrutil.cc:692-699)
    cx<double> em = ep * m;
    double rr = std::sqrt(std::hypot(em.re, em.im));
    double th = 0.5 * std::atan2(em.im, em.re);
    cx<double> rt = cxd(rr * std::cos(th), rr * std::sin(th));
    if (rt.im < 0) rt = cxd(-rt.re, -rt.im);
    cx<double> k = rt * omega;
    ra.k[r] = k;
    cx<double> I = cxd(0.0, 1.0);
    double sg = b.sign[r];
    ra.pf1[r] = sg * (I * m * omega);
    cx<double> pf2 = (-sg) * (I * k);
    ra.pfc[r] = (k.re == 0.0 && k.im == 0.0) ? cxd(0.0, 0.0) : cdiv(pf2, I * k);
    ra.pf3[r] = (-sg) * (I * ep * omega);
  }
  return ra;
}

// One region's contribution with the signs of an exterior region
// (KK = i mu w GC0, KN = NK = -i k GC1, NN = -i eps w GC0): the matrix of the
// EMT power's quadratic form.  nreg = 0 when the block does not see region R.
static RegionArgs single_region_args(const Block& b, const RegionArgs& ra, int R, double wr, double wi,
                                     const double* eps, const double* mu) {
  RegionArgs rb;
  memset(&rb, 0, sizeof rb);
  for (int r = 0; r < ra.nreg; r++) {
    if (b.reg[r] != R) continue;
    const cx<double> I = cxd(0.0, 1.0), w = cxd(wr, wi);
    rb.k[0] = ra.k[r];
    rb.pf1[0] = I * cxd(mu[2 * R], mu[2 * R + 1]) * w;
    rb.pfc[0] = cxd(-1.0, 0.0);
    rb.pf3[0] = (-1.0) * (I * cxd(eps[2 * R], eps[2 * R + 1]) * w);
    rb.nreg = 1;
  }
  return rb;
}

gbem_status assemble_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int precision,
                            void* dM, int ld, int dtype, cudaStream_t s, const BlockSel* only, int only_region) {
  if ((precision == GBEM_PREC_FP64 && dtype != GBEM_C128) || (precision == GBEM_PREC_MIXED && dtype != GBEM_C64)) {
    set_error("gbem_assemble: matrix dtype does not match the precision (C128 for FP64, C64 for MIXED)");
    return GBEM_EINVAL;
  }
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  if (!g->fippi_ready) {
    st = compute_fippi(g, s);
    if (st != GBEM_OK) return st;
  }
  bool any_empty = only_region >= 0;  // a single region leaves blocks without it at zero
  for (const Block& b : g->blocks)
    if (!only || (b.sa == std::min(only->nsa, only->nsb) && b.sb == std::max(only->nsa, only->nsb)))
      any_empty |= (b.nreg == 0);
  size_t esz = dtype == GBEM_C128 ? 16 : 8;
  if (any_empty) {
    // surfaces that share no region interact with zero: clear what is written
    cudaError_t e;
    if (!only) {
      e = cudaMemset2DAsync(dM, (size_t)ld * esz, 0, (size_t)g->N * esz, g->N, s);
    } else {
      const int na = g->S[only->nsa].ne * (g->S[only->nsa].pec ? 1 : 2);
      const int nb = g->S[only->nsb].ne * (g->S[only->nsb].pec ? 1 : 2);
      e = cudaMemset2DAsync((char*)dM + ((size_t)only->row0 + (size_t)only->col0 * ld) * esz, (size_t)ld * esz, 0,
                            (size_t)na * esz, nb, s);
    }
    if (e != cudaSuccess) return cuda_status(e, "memset matrix");
  }
  int* d_status = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&d_status, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e, "status word");
  for (size_t bi = 0; bi < g->blocks.size(); bi++) {
    const Block& b = g->blocks[bi];
    DevBlock* db = g->dblocks[bi];
    if (b.nreg == 0) continue;
    if (only && !(b.sa == std::min(only->nsa, only->nsb) && b.sb == std::max(only->nsa, only->nsb))) continue;
    RegionArgs ra = region_args(b, wr, wi, eps, mu);
    if (only_region >= 0) {
      ra = single_region_args(b, ra, only_region, wr, wi, eps, mu);
      if (ra.nreg == 0) continue;
    }
    {
      StatTimer tn(ST_NEAR, s);
      if (db->nself) {
        stats_launch(ST_NEAR);
        self_kernel<<<(db->nself + 3) / 4, 128, 0, s>>>(db->near, db->self_list, db->nself, g->d_pv, ra, db->nearval);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "self_kernel");
      }
      if (db->nother) {
        stats_launch(ST_NEAR);
        near_kernel<<<(db->nother + 63) / 64, 64, 0, s>>>(db->near, db->other_list, db->nother, g->d_pv, db->fippi,
                                                          ra, db->nearval, d_status);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "near_kernel");
        // touching pairs in the short-wavelength regime (only when some k |r| can exceed pi)
        double kmax = 0.0;
        for (int r = 0; r < b.nreg; r++) kmax = std::fmax(kmax, std::hypot(ra.k[r].re, ra.k[r].im));
        if (kmax * b.rmax_touch > M_PI) {
          stats_launch(ST_NEAR);
          td_touch_kernel<<<(db->nother + 3) / 4, 128, 0, s>>>(db->near, db->other_list, db->nother, g->d_pv, ra,
                                                               db->nearval);
          if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "td_touch_kernel");
        }
      }
    }
    TileArgs ta;
    ta.rows = db->rows; ta.cols = db->cols; ta.tiles = db->tiles;
    ta.pv = g->d_pv; ta.pc = g->d_pc; ta.elen_a = db->elen_a; ta.elen_b = db->elen_b;
    ta.nptr = db->nptr; ta.ncol = db->ncol; ta.nidx = db->nidx; ta.nearval = db->nearval;
    ta.row_panel_offset = g->S[b.sa].panel_offset;
    ta.bpe_a = b.bpe_a; ta.bpe_b = b.bpe_b;
    ta.row_off = g->S[b.sa].bf_offset; ta.col_off = g->S[b.sb].bf_offset;
    ta.mrow_off = ta.col_off; ta.mcol_off = ta.row_off;
    ta.passes = 3;
    if (only) {
      // block assembly: the (nsa, nsb) block at (row0, col0) of dM
      if (b.sa == only->nsa) {
        ta.row_off = only->row0; ta.col_off = only->col0;
        ta.mrow_off = only->row0; ta.mcol_off = only->col0;  // a self block mirrors into itself
        ta.passes = b.sym ? 3 : 1;
      } else {
        ta.mrow_off = only->row0; ta.mcol_off = only->col0;  // (nsa, nsb) is the mirror of (sb, sa)
        ta.passes = 2;
      }
    }
    ta.sym = b.sym ? 1 : 0;
    ta.out = dM; ta.ld = ld;
    int nc = (b.bpe_a == 2 && b.bpe_b == 2) ? 3 : ((b.bpe_a == 1 && b.bpe_b == 1) ? 1 : 2);
    StatTimer tf(ST_FAR, s);
    if (precision != GBEM_PREC_MIXED) stats_launch(ST_FAR);
    if (precision == GBEM_PREC_MIXED) {
      e = nc == 1 ? far_mixed<1>(g, b, db, ta, ra, s) : nc == 2 ? far_mixed<2>(g, b, db, ta, ra, s) : far_mixed<3>(g, b, db, ta, ra, s);
    } else {
      e = nc == 1 ? launch_tiles64<1>(ta, ra, db->ntiles, s)
                  : nc == 2 ? launch_tiles64<2>(ta, ra, db->ntiles, s) : launch_tiles64<3>(ta, ra, db->ntiles, s);
    }
    if (e != cudaSuccess) return cuda_status(e, "tile_kernel");
  }
  int h_status = 0;
  e = cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaFreeAsync(d_status, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e, "assembly");
  if (h_status) {
    set_error("touching panel pairs in the short-wavelength regime (|k r| > pi) need the full-kernel "
              "Taylor-Duffy path, which this build does not implement");
    return GBEM_ENOTSUP;
  }
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// Gradient blocks dM/dx_mu of one surface block (AssembleBEMMatrixBlock with
// GradM, the scuff-cas3D force path): one thread per edge pair, the four
// panel pairs integrated directly with the reference's gradient integrand
// (PanelPanelInteractions.cc:166-181):
//   GradH[2mu]   = int int R_mu hPlus Psi,
//   GradH[2mu+1] = int int (R_mu hTimes Zeta + (F x F')_mu Psi),
// hPlus = F.F' - 4/k^2, hTimes = (F x F').R, Zeta = Phi (-k^2 - 3ik/r + 3/r^2)/r^2.
// Rules as the reference chooses them: far pairs (rRel > 4) the 6x6 rule;
// near pairs the high-order rule without desingularisation; pairs that take
// the Taylor-Duffy branch (ncv = 3, or ncv > 0 when |k r| > pi) contribute
// zero (PanelPanelInteractions.cc:488).  Stamped like GC (GradGC[1] carries
// the 1/(ik) of GC[1]).
// ---------------------------------------------------------------------------
struct GradArgs {
  const double* V;   // vertices of both surfaces' panels: global panel vertex table (9 per panel)
  const double* pc;  // centroid + radius per global panel
  const int* Ea;     // 8 ints per edge of surface a
  const int* Eb;
  const double* La;  // edge lengths
  const double* Lb;
  int nea, neb, poff_a, poff_b;  // edges; first global panel index of each surface
  const double* Va;  // vertex arrays of the two surfaces (for the Q vertices)
  const double* Vb;
  int bpe_a, bpe_b;
  int row0, col0;
  long long ld;
  void* out[3];      // dM/dx_mu (null: not wanted)
  int nta;           // rotation axes (0..3)
  double gamma[27];  // per axis: dX = Gamma X, Gamma[9 a + mu + 3 nu] (GammaMatrix of AssembleBEMMatrixBlock)
  void* outT[3];     // dM/dtheta_a
};

// TH (2 per axis, may be null): the angular derivatives of the reference
// (PanelPanelInteractions.cc:183-199): with dX = Gamma x, dF = Gamma F,
//   dHdT[2a]   = int int hPlus (R.dX) Psi + (dF.F') Phi,
//   dHdT[2a+1] = int int hTimes (R.dX) Zeta + ((dF x F').R + (F x F').dX) Psi.
__device__ void ppi_grad(const double* Pa, const double* Qa, const double* Pb, const double* Qb, cx<double> k,
                         const double* rule, int npts, cx<double>* GH, int nta = 0, const double* gamma = nullptr,
                         cx<double>* TH = nullptr) {
  const double inv4pi = 0.079577471545947667884;
  const cx<double> ik = mk(-k.im, k.re), ik2 = ik * ik, m4 = cdiv(mk(4.0, 0.0), ik2);
  double A[3], B[3], Ap[3], Bp[3];
  for (int c = 0; c < 3; c++) {
    A[c] = Pa[3 + c] - Pa[c]; B[c] = Pa[6 + c] - Pa[c];
    Ap[c] = Pb[3 + c] - Pb[c]; Bp[c] = Pb[6 + c] - Pb[c];
  }
  for (int m = 0; m < 6; m++) GH[m] = mk(0.0, 0.0);
  for (int m = 0; m < 2 * nta; m++) TH[m] = mk(0.0, 0.0);
  for (int i = 0; i < npts; i++) {
    const double u = rule[3 * i], v = rule[3 * i + 1], wi = rule[3 * i + 2];
    double x[3], F[3];
    for (int c = 0; c < 3; c++) { x[c] = Pa[c] + u * A[c] + v * B[c]; F[c] = x[c] - Qa[c]; }
    for (int j = 0; j < npts; j++) {
      const double up = rule[3 * j], vp = rule[3 * j + 1], wj = rule[3 * j + 2];
      double xp[3], Fp[3], R[3];
      for (int c = 0; c < 3; c++) {
        xp[c] = Pb[c] + up * Ap[c] + vp * Bp[c];
        Fp[c] = xp[c] - Qb[c];
        R[c] = x[c] - xp[c];
      }
      const double r2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2], r = sqrt(r2), ri = 1.0 / r;
      double sn, cs;
      sincos(k.re * r, &sn, &cs);
      const double amp = wi * wj * inv4pi * ri * exp(-k.im * r);
      const cx<double> Phi = mk(amp * cs, amp * sn);
      const cx<double> Psi = Phi * mk(ik.re - ri, ik.im) * mk(ri, 0.0);
      const cx<double> Zeta = Phi * (ik2 - mk(3.0 * ri, 0.0) * ik + mk(3.0 * ri * ri, 0.0)) * mk(ri * ri, 0.0);
      const cx<double> hPlus = mk(F[0] * Fp[0] + F[1] * Fp[1] + F[2] * Fp[2], 0.0) + m4;
      double X[3];
      vcross(F, Fp, X);
      const double hT = X[0] * R[0] + X[1] * R[1] + X[2] * R[2];
      const cx<double> hPsi = hPlus * Psi;
      const cx<double> hZ = hT * Zeta;
      for (int mu = 0; mu < 3; mu++) {
        GH[2 * mu] = GH[2 * mu] + R[mu] * hPsi;
        GH[2 * mu + 1] = GH[2 * mu + 1] + R[mu] * hZ + X[mu] * Psi;
      }
      for (int a = 0; a < nta; a++) {
        const double* Gm = gamma + 9 * a;
        double dX[3], dF[3], dFxFp[3];
        for (int mu = 0; mu < 3; mu++) {
          dX[mu] = Gm[mu] * x[0] + Gm[mu + 3] * x[1] + Gm[mu + 6] * x[2];
          dF[mu] = Gm[mu] * F[0] + Gm[mu + 3] * F[1] + Gm[mu + 6] * F[2];
        }
        vcross(dF, Fp, dFxFp);
        const double Puv = R[0] * dX[0] + R[1] * dX[1] + R[2] * dX[2];
        const double dFFp = dF[0] * Fp[0] + dF[1] * Fp[1] + dF[2] * Fp[2];
        const double cr = dFxFp[0] * R[0] + dFxFp[1] * R[1] + dFxFp[2] * R[2] + X[0] * dX[0] + X[1] * dX[1] + X[2] * dX[2];
        TH[2 * a] = TH[2 * a] + Puv * hPsi + dFFp * Phi;
        TH[2 * a + 1] = TH[2 * a + 1] + Puv * hZ + cr * Psi;
      }
    }
  }
}

template <bool REAL>
__global__ void __launch_bounds__(128) grad_kernel(GradArgs a, RegionArgs ra) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.nea * a.neb) return;
  const int ea = (int)(t % a.nea), eb = (int)(t / a.nea);
  const int* EA = a.Ea + 8 * ea;
  const int* EB = a.Eb + 8 * eb;
  const double La = a.La[ea], Lb = a.Lb[eb];
  cx<double> acc[3][4], accT[3][4];
  for (int mu = 0; mu < 3; mu++)
    for (int c = 0; c < 4; c++) acc[mu][c] = accT[mu][c] = mk(0.0, 0.0);
  for (int r = 0; r < ra.nreg; r++) {
    const cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    cx<double> S0[3], S1[3], T0[3], T1[3];
    for (int mu = 0; mu < 3; mu++) S0[mu] = S1[mu] = T0[mu] = T1[mu] = mk(0.0, 0.0);
    for (int sa = 0; sa < 2; sa++) {
      const int iqa = sa == 0 ? EA[2] : EA[3];
      const int pa = sa == 0 ? EA[4] : EA[5];
      if (iqa < 0 || pa < 0) continue;
      for (int sb = 0; sb < 2; sb++) {
        const int iqb = sb == 0 ? EB[2] : EB[3];
        const int pb = sb == 0 ? EB[4] : EB[5];
        if (iqb < 0 || pb < 0) continue;
        const int gpa = a.poff_a + pa, gpb = a.poff_b + pb;
        const double* Pa = a.V + 9 * (size_t)gpa;
        const double* Pb = a.V + 9 * (size_t)gpb;
        const double* ca = a.pc + 4 * (size_t)gpa;
        const double* cb = a.pc + 4 * (size_t)gpb;
        const double rmax = fmax(ca[3], cb[3]);
        const double dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
        const bool far = sqrt(dx * dx + dy * dy + dz * dz) > 4.0 * rmax;
        cx<double> GH[6], TH[6];
        if (far) {
          ppi_grad(Pa, a.Va + 3 * iqa, Pb, a.Vb + 3 * iqb, k, c_lo64, 6, GH, a.nta, a.gamma, TH);
        } else {
          int ncv = 0;
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
              const double ex = Pa[3 * i] - Pb[3 * j], ey = Pa[3 * i + 1] - Pb[3 * j + 1], ez = Pa[3 * i + 2] - Pb[3 * j + 2];
              if (sqrt(ex * ex + ey * ey + ez * ez) < 1e-6 * rmax) ncv++;
            }
          const bool swr = hypot(k.re * rmax, k.im * rmax) > M_PI;
          if (ncv == 3 || (ncv > 0 && swr)) continue;  // Taylor-Duffy pairs: zero gradient
          ppi_grad(Pa, a.Va + 3 * iqa, Pb, a.Vb + 3 * iqb, k, c_ho, HO_N * HO_N, GH, a.nta, a.gamma, TH);
        }
        const double sg = (sa == sb) ? 1.0 : -1.0;
        for (int mu = 0; mu < 3; mu++) {
          S0[mu] = S0[mu] + sg * GH[2 * mu];
          S1[mu] = S1[mu] + sg * GH[2 * mu + 1];
        }
        for (int t = 0; t < a.nta; t++) {
          T0[t] = T0[t] + sg * TH[2 * t];
          T1[t] = T1[t] + sg * TH[2 * t + 1];
        }
      }
    }
    const double LL = La * Lb;
    for (int mu = 0; mu < 3; mu++) {
      const cx<double> g0 = LL * S0[mu], g1 = LL * S1[mu];
      acc[mu][0] = acc[mu][0] + ra.pf1[r] * g0;
      acc[mu][1] = acc[mu][1] + ra.pfc[r] * g1;
      acc[mu][3] = acc[mu][3] + ra.pf3[r] * g0;
    }
    for (int t = 0; t < a.nta; t++) {  // stamped like the gradient (SurfaceSurfaceInteractions.cc:216-325)
      const cx<double> g0 = LL * T0[t], g1 = LL * T1[t];
      accT[t][0] = accT[t][0] + ra.pf1[r] * g0;
      accT[t][1] = accT[t][1] + ra.pfc[r] * g1;
      accT[t][3] = accT[t][3] + ra.pf3[r] * g0;
    }
  }
  const long long X = a.row0 + (long long)a.bpe_a * ea, Y = a.col0 + (long long)a.bpe_b * eb;
  for (int m = 0; m < 6; m++) {
    const int mu = m % 3;
    void* dst = m < 3 ? a.out[mu] : (mu < a.nta ? a.outT[mu] : nullptr);
    if (!dst) continue;
    const cx<double>* v = m < 3 ? acc[mu] : accT[mu];
    // (K,K) = PF1 G0; (K,N) = (N,K) = PF2 G1 / (ik); (N,N) = PF3 G0
    cx<double> e[2][2] = {{v[0], v[1]}, {v[1], v[3]}};
    for (int dx = 0; dx < a.bpe_a; dx++)
      for (int dy = 0; dy < a.bpe_b; dy++) {
        const long long idx = (X + dx) + (Y + dy) * a.ld;
        if (REAL) ((double*)dst)[idx] = e[dx][dy].re;
        else ((cx<double>*)dst)[idx] = e[dx][dy];
      }
  }
}

gbem_status assemble_gradient_device(Geometry* g, double wr, double wi, const double* eps, const double* mu,
                                     const BlockSel& sel, void* const out[3], int ld, int dtype, cudaStream_t s,
                                     int nta, const double* gamma, void* const* outT) {
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  const int lo = std::min(sel.nsa, sel.nsb), hi = std::max(sel.nsa, sel.nsb);
  const Block* bp = nullptr;
  for (const Block& b : g->blocks)
    if (b.sa == lo && b.sb == hi) bp = &b;
  if (!bp) { set_error("gradient: no such surface block"); return GBEM_EINVAL; }
  const Surface& A = g->S[sel.nsa];
  const Surface& B = g->S[sel.nsb];
  const size_t es = dtype == GBEM_F64 ? 8 : 16;
  cudaError_t e = cudaSuccess;
  // the block's entries are written by one thread each; a block of surfaces
  // that share no region is zero
  for (int m = 0; m < 6 && e == cudaSuccess; m++) {
    void* dst = m < 3 ? out[m] : (m - 3 < nta ? outT[m - 3] : nullptr);
    if (dst)
      e = cudaMemset2DAsync((char*)dst + ((size_t)sel.row0 + (size_t)sel.col0 * ld) * es, (size_t)ld * es, 0,
                            (size_t)A.ne * (A.pec ? 1 : 2) * es, B.ne * (B.pec ? 1 : 2), s);
  }
  if (e != cudaSuccess) return cuda_status(e, "gradient memset");
  if (bp->nreg == 0 || A.ne == 0 || B.ne == 0) return GBEM_OK;
  double *dVa = nullptr, *dVb = nullptr, *dLa = nullptr, *dLb = nullptr;
  int *dEa = nullptr, *dEb = nullptr;
  e = dupload(&dVa, A.V.data(), A.V.size());
  if (e == cudaSuccess) e = dupload(&dVb, B.V.data(), B.V.size());
  if (e == cudaSuccess) e = dupload(&dEa, A.E.data(), A.E.size());
  if (e == cudaSuccess) e = dupload(&dEb, B.E.data(), B.E.size());
  if (e == cudaSuccess) e = dupload(&dLa, A.elen.data(), A.elen.size());
  if (e == cudaSuccess) e = dupload(&dLb, B.elen.data(), B.elen.size());
  if (e == cudaSuccess) {
    GradArgs ga;
    ga.V = g->d_pv; ga.pc = g->d_pc; ga.Ea = dEa; ga.Eb = dEb; ga.La = dLa; ga.Lb = dLb;
    ga.nea = A.ne; ga.neb = B.ne; ga.poff_a = A.panel_offset; ga.poff_b = B.panel_offset;
    ga.Va = dVa; ga.Vb = dVb;
    ga.bpe_a = A.pec ? 1 : 2; ga.bpe_b = B.pec ? 1 : 2;
    ga.row0 = sel.row0; ga.col0 = sel.col0; ga.ld = ld;
    for (int m = 0; m < 3; m++) ga.out[m] = out[m];
    ga.nta = nta;
    for (int m = 0; m < 27; m++) ga.gamma[m] = m < 9 * nta ? gamma[m] : 0.0;
    for (int m = 0; m < 3; m++) ga.outT[m] = m < nta ? outT[m] : nullptr;
    const RegionArgs ra = region_args(*bp, wr, wi, eps, mu);
    const long long n = (long long)A.ne * B.ne;
    stats_launch(ST_OTHER);
    if (dtype == GBEM_F64) grad_kernel<true><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(ga, ra);
    else grad_kernel<false><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(ga, ra);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  cudaFree(dVa); cudaFree(dVb); cudaFree(dEa); cudaFree(dEb); cudaFree(dLa); cudaFree(dLb);
  return cuda_status(e, "gradient block");
}

// ---------------------------------------------------------------------------
// plane-wave right-hand side (AssembleRHSVector.cc:145-255, 288-340 with a
// PlaneWave source in the exterior region, libs/libIncField/PlaneWave.cc:71-87)
//   K entry: -<f_n, E_inc>/ZVAC,  N entry: -<f_n, H_inc>  (dielectric surfaces)
// ---------------------------------------------------------------------------
struct RhsArgs {
  const double* V;  // surface vertices
  const int* E;     // 8 ints per edge
  const double* elen;
  int ne, bf_offset, pec, sign;  // sign: -1 incident field outside, +1 inside
  cx<double> k, Z;               // wavenumber and wave impedance of the source region
  cx<double> E0[3];
  double nh[3];
  cx<double>* rhs;
};

__device__ void pw_fields(const RhsArgs& a, const double* X, cx<double>* Ef, cx<double>* Hf) {
  double ph = a.nh[0] * X[0] + a.nh[1] * X[1] + a.nh[2] * X[2];
  cx<double> ex = cexpo(mk(-a.k.im * ph, a.k.re * ph));
  for (int i = 0; i < 3; i++) Ef[i] = a.E0[i] * ex;
  Hf[0] = cdiv(a.nh[1] * Ef[2] - a.nh[2] * Ef[1], a.Z);
  Hf[1] = cdiv(a.nh[2] * Ef[0] - a.nh[0] * Ef[2], a.Z);
  Hf[2] = cdiv(a.nh[0] * Ef[1] - a.nh[1] * Ef[0], a.Z);
}

__global__ void rhs_kernel(RhsArgs a) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne) return;
  const int* ed = a.E + 8 * e;
  const double* V1 = a.V + 3 * ed[0];
  const double* V2 = a.V + 3 * ed[1];
  cx<double> Ep = mk(0.0, 0.0), Hp = mk(0.0, 0.0);
  for (int side = 0; side < 2; side++) {
    int iq = side == 0 ? ed[2] : ed[3];
    if (iq < 0) continue;
    const double* Q = a.V + 3 * iq;
    double A[3], B[3];
    for (int i = 0; i < 3; i++) { A[i] = V1[i] - Q[i]; B[i] = V2[i] - Q[i]; }
    cx<double> se = mk(0.0, 0.0), sh = mk(0.0, 0.0);
    for (int q = 0; q < HO_N * HO_N; q++) {
      double u = c_ho[3 * q], v = c_ho[3 * q + 1], w = c_ho[3 * q + 2];
      double X[3], F[3];
      for (int i = 0; i < 3; i++) { F[i] = u * A[i] + v * B[i]; X[i] = Q[i] + F[i]; }
      cx<double> Ef[3], Hf[3];
      pw_fields(a, X, Ef, Hf);
      for (int i = 0; i < 3; i++) { se = se + (w * F[i]) * Ef[i]; sh = sh + (w * F[i]) * Hf[i]; }
    }
    // (L/2A) int (X-Q).E dA = L int_std (X-Q).E
    double L = a.elen[e];
    if (side == 0) { Ep = Ep + L * se; Hp = Hp + L * sh; }
    else { Ep = Ep - L * se; Hp = Hp - L * sh; }
  }
  const double ZVAC = 376.73031346177;
  double sg = (double)a.sign;
  if (a.pec) a.rhs[a.bf_offset + e] = (sg / ZVAC) * Ep;
  else {
    a.rhs[a.bf_offset + 2 * e] = (sg / ZVAC) * Ep;
    a.rhs[a.bf_offset + 2 * e + 1] = sg * Hp;
  }
}

gbem_status rhs_planewave_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, const double* E0,
                                 const double* nh, void* d_rhs, cudaStream_t s) {
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  cudaError_t e = cudaMemsetAsync(d_rhs, 0, sizeof(double) * 2 * g->N, s);
  if (e != cudaSuccess) return cuda_status(e, "rhs memset");
  for (Surface& S : g->S) {
    // the incident field lives in region 0 (the exterior medium)
    int sign;
    if (S.reg_ext == 0) sign = -1;
    else if (S.reg_int == 0) sign = 1;
    else continue;
    RhsArgs a;
    double *dV = nullptr, *dL = nullptr;
    int* dE = nullptr;
    e = dupload(&dV, S.V.data(), S.V.size());
    if (e == cudaSuccess) e = dupload(&dE, S.E.data(), S.E.size());
    if (e == cudaSuccess) e = dupload(&dL, S.elen.data(), S.elen.size());
    if (e != cudaSuccess) return cuda_status(e, "rhs upload");
    a.V = dV; a.E = dE; a.elen = dL; a.ne = S.ne; a.bf_offset = S.bf_offset; a.pec = S.pec ? 1 : 0; a.sign = sign;
    cx<double> ep = cxd(eps[0], eps[1]), m = cxd(mu[0], mu[1]), em = ep * m;
    double rr = std::sqrt(std::hypot(em.re, em.im)), th = 0.5 * std::atan2(em.im, em.re);
    cx<double> rt = cxd(rr * std::cos(th), rr * std::sin(th));  // principal sqrt, as std::sqrt
    a.k = rt * cxd(wr, wi);
    cx<double> q = cdiv(m, ep);
    double rq = std::sqrt(std::hypot(q.re, q.im)), tq = 0.5 * std::atan2(q.im, q.re);
    a.Z = 376.73031346177 * cxd(rq * std::cos(tq), rq * std::sin(tq));
    for (int i = 0; i < 3; i++) { a.E0[i] = cxd(E0[2 * i], E0[2 * i + 1]); a.nh[i] = nh[i]; }
    a.rhs = (cx<double>*)d_rhs;
    if (S.ne) rhs_kernel<<<(S.ne + 127) / 128, 128, 0, s>>>(a);
    e = cudaGetLastError();
    cudaStreamSynchronize(s);
    cudaFree(dV); cudaFree(dE); cudaFree(dL);
    if (e != cudaSuccess) return cuda_status(e, "rhs_kernel");
  }
  return GBEM_OK;
}

// ---------------------------------------------------------------------------
// Adjoint contraction with the vertex derivatives of the matrix and of the
// plane-wave right-hand side (no reference counterpart: the reference
// differentiates rigid motions of whole surfaces only, GradM / dMdT).
//   grad[3 v + c] = Re sum_r sum_ij conj(lam_ir) dM_ij/dV_vc x_jr
// The matrix derivative is never formed: every panel pair adds its share to
// the vertex gradients directly.
//  vjp_far_kernel   far pairs (rRel > 4), one thread per pair: reverse-mode
//                   derivative of the 6x6-rule integrals (adjoint.cuh), the
//                   edge-length factors La Lb included.
//  vjp_near_kernel  near and common-vertex pairs, one warp per (pair,
//                   vertex, coordinate) -- one vertex per pair follows from
//                   translation invariance: central differences of the FP64
//                   near-pair evaluation (static integrals recomputed for the
//                   displaced vertices), contracted with the same weights.
//  rhs_vjp_kernel   Re sum conj(g_i) db_i/dV for plane-wave right-hand sides.
// ---------------------------------------------------------------------------
struct VjpTables {
  const double* pv;   // 9 per global panel: vertices in mesh order
  const double* pc;   // 4 per global panel: centroid, radius
  const int* pvi;     // 3 per global panel: global vertex indices
  const int* sbf;     // 3 per global panel: basis function of the edge whose Q is vertex j (-1: none)
  const double* ssl;  // 3 per global panel: +L on the edge's positive panel, -L on its negative one
  const cx<double>* lam;
  const cx<double>* x;
  long long ldl, ldx;
  int nrhs;
  double* grad;       // 3 per global vertex
};

__device__ __forceinline__ cx<double> conj_mul(cx<double> a, cx<double> b) {
  return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}

// W[ch][3 ja + jb]: sum over the right-hand sides of conj(lam_i) x_j for the
// entry (i, j) of the (Qa, Qb) edge pair, plus its mirror (j, i) when the
// pair stands for both orders; channel 0 = (E, E), 1 = (E, H) + (H, E),
// 2 = (H, H) (the (K, K), (K, N), (N, N) entries of SurfaceSurfaceInteractions.cc:205-327)
__device__ void vjp_weights(const VjpTables& t, int gpa, int gpb, int bpe_a, int bpe_b, bool mirror, cx<double> W[3][9]) {
  for (int ch = 0; ch < 3; ch++)
    for (int m = 0; m < 9; m++) W[ch][m] = mk(0.0, 0.0);
  for (int ja = 0; ja < 3; ja++) {
    const int ia = t.sbf[3 * gpa + ja];
    if (ia < 0) continue;
    for (int jb = 0; jb < 3; jb++) {
      const int ib = t.sbf[3 * gpb + jb];
      if (ib < 0) continue;
      for (int r = 0; r < t.nrhs; r++) {
        const cx<double>* L = t.lam + (long long)r * t.ldl;
        const cx<double>* X = t.x + (long long)r * t.ldx;
        for (int al = 0; al < bpe_a; al++)
          for (int bt = 0; bt < bpe_b; bt++) {
            const int ch = (al == 0 && bt == 0) ? 0 : (al != bt ? 1 : 2);
            cx<double> w = conj_mul(L[ia + al], X[ib + bt]);
            if (mirror) w = w + conj_mul(L[ib + bt], X[ia + al]);
            W[ch][3 * ja + jb] = W[ch][3 * ja + jb] + w;
          }
      }
    }
  }
}

// the three channels of vjp_weights for one (Qa, Qb) combination m = 3 ja + jb
// (one lane each in the warp-per-pair adjoint kernel)
__device__ void vjp_weights_m(const VjpTables& t, int gpa, int gpb, int bpe_a, int bpe_b, bool mirror, int m,
                              cx<double>* w3) {
  w3[0] = w3[1] = w3[2] = mk(0.0, 0.0);
  const int ia = t.sbf[3 * gpa + m / 3], ib = t.sbf[3 * gpb + m % 3];
  if (ia < 0 || ib < 0) return;
  for (int r = 0; r < t.nrhs; r++) {
    const cx<double>* L = t.lam + (long long)r * t.ldl;
    const cx<double>* X = t.x + (long long)r * t.ldx;
    for (int al = 0; al < bpe_a; al++)
      for (int bt = 0; bt < bpe_b; bt++) {
        const int ch = (al == 0 && bt == 0) ? 0 : (al != bt ? 1 : 2);
        cx<double> w = conj_mul(L[ia + al], X[ib + bt]);
        if (mirror) w = w + conj_mul(L[ib + bt], X[ia + al]);
        w3[ch] = w3[ch] + w;
      }
  }
}

struct VjpFarArgs {
  VjpTables t;
  int offa, offb, npa, npb, bpe_a, bpe_b, sym;
};

// grid (column panels / 128, row panels): one far pair per thread; the row
// panel's gradient is reduced over each warp before its atomics
__global__ void __launch_bounds__(128) vjp_far_kernel(VjpFarArgs a, RegionArgs ra) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  const int gpa = a.offa + i, gpb = a.offb + j;
  const VjpTables& t = a.t;
  double gA[9], gB[9];
  for (int q = 0; q < 9; q++) gA[q] = gB[q] = 0.0;
  bool act = j < a.npb && !(a.sym && j <= i);
  if (act) act = is_far(t.pc + 4 * (size_t)gpa, t.pc + 4 * (size_t)gpb, t.pc[4 * (size_t)gpa + 3], t.pc[4 * (size_t)gpb + 3]);
  if (act) {
    double Va[9], Vb[9], slA[3], slB[3];
    for (int q = 0; q < 9; q++) { Va[q] = t.pv[9 * (size_t)gpa + q]; Vb[q] = t.pv[9 * (size_t)gpb + q]; }
    for (int q = 0; q < 3; q++) {
      slA[q] = t.sbf[3 * gpa + q] >= 0 ? t.ssl[3 * gpa + q] : 0.0;
      slB[q] = t.sbf[3 * gpb + q] >= 0 ? t.ssl[3 * gpb + q] : 0.0;
    }
    cx<double> W[3][9];
    vjp_weights(t, gpa, gpb, a.bpe_a, a.bpe_b, true, W);
    double ErT[3] = {0.0, 0.0, 0.0}, EcT[3] = {0.0, 0.0, 0.0};
    for (int r = 0; r < ra.nreg; r++) {
      const cx<double> k = ra.k[r];
      if (k.re == 0.0 && k.im == 0.0) continue;
      cx<double> C0[9], C1[9];
      for (int m = 0; m < 9; m++) {
        const double fac = slA[m / 3] * slB[m % 3];
        C0[m] = fac * (ra.pf1[r] * W[0][m] + ra.pf3[r] * W[2][m]);
        C1[m] = fac * (ra.pfc[r] * W[1][m]);
      }
      double Er[3], Ec[3];
      far_pair_vjp(Va, Vb, k, C0, C1, c_lo64, 6, gA, gB, Er, Ec);
      for (int q = 0; q < 3; q++) { ErT[q] += Er[q]; EcT[q] += Ec[q]; }
    }
    // the coefficients hold La Lb: d/dL = (slot sum)/L, dL/dV along the edge
    for (int q = 0; q < 3; q++) {
      const int q1 = (q + 1) % 3, q2 = (q + 2) % 3;
      if (slA[q] != 0.0) {
        const double s = ErT[q] / (slA[q] * slA[q]);
        for (int c = 0; c < 3; c++) {
          const double d = Va[3 * q1 + c] - Va[3 * q2 + c];
          gA[3 * q1 + c] += s * d; gA[3 * q2 + c] -= s * d;
        }
      }
      if (slB[q] != 0.0) {
        const double s = EcT[q] / (slB[q] * slB[q]);
        for (int c = 0; c < 3; c++) {
          const double d = Vb[3 * q1 + c] - Vb[3 * q2 + c];
          gB[3 * q1 + c] += s * d; gB[3 * q2 + c] -= s * d;
        }
      }
    }
    for (int q = 0; q < 9; q++)
      if (gB[q] != 0.0) atomicAdd(&t.grad[3 * (size_t)t.pvi[3 * gpb + q / 3] + q % 3], gB[q]);
  }
  for (int q = 0; q < 9; q++) {
    double v = gA[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffff, v, o);
    if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&t.grad[3 * (size_t)t.pvi[3 * gpa + q / 3] + q % 3], v);
  }
}

// Re sum over regions and (Qa, Qb) of the pair's weighted values at the given
// vertex positions -- the arithmetic of self_kernel, near_kernel and
// td_touch_kernel for one pair by one warp (the static integrals at the
// adjoint's 8-point rule; the point sums of the static integrals, of the
// self and touching Helmholtz integrals dealt to the lanes and reduced), with
// the edge lengths taken from the positions.  Every lane returns the value.
__device__ double near_pair_energy(const DevNear& d, const double* Va, const double* Vb, const double* sgA,
                                   const double* sgB, const RegionArgs& ra, const cx<double> (*W)[9], int lane,
                                   const double* sgx8, const double* sgw8, const double* srule6,
                                   const double* srule16) {
  const bool self = d.pa == d.pb;
  // lane m < 9 forms the (Qa, Qb) combination m = 3 ja + jb; the sums over
  // cubature points before it are spread over all lanes
  const int m = lane < 9 ? lane : 0;
  const int ja = m / 3, jb = m % 3;
  double fac;
  {
    double La = 0.0, Lb = 0.0;
    for (int c = 0; c < 3; c++) {
      const double ea = Va[3 * ((ja + 1) % 3) + c] - Va[3 * ((ja + 2) % 3) + c];
      const double eb = Vb[3 * ((jb + 1) % 3) + c] - Vb[3 * ((jb + 2) % 3) + c];
      La += ea * ea; Lb += eb * eb;
    }
    fac = sgA[ja] * sgB[jb] * sqrt(La) * sqrt(Lb);
  }
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  Fippi F;
  bool haveF = false;
  double E = 0.0;
  for (int r = 0; r < ra.nreg; r++) {
    const cx<double> k = ra.k[r];
    if (k.re == 0.0 && k.im == 0.0) continue;
    const cx<double> m4ok2 = cdiv(mk(-4.0, 0.0), k * k);
    cx<double> H0, H1;
    if (self) {
      cx<double> MG[9], MP[9];
      self_moments(Va, k, srule16, srule16 + NT_SELF, NT_SELF, MG, lane, 32);
      cx_warp_sum(MG, 9);
      for (int q = 0; q < 9; q++) MP[q] = mk(0.0, 0.0);
      double c[9], dd[9];
      combo_coeffs(Va, Va, ja, jb, c, dd);
      combine(MG, MP, c, dd, m4ok2, &H0, &H1);
      H1 = mk(0.0, 0.0);
    } else {
      const bool sw = hypot(k.re * d.rmax, k.im * d.rmax) > M_PI;
      cx<double> MG[9], MP[9];
      bool desing = false, td = false;
      cx<double> T[10];
      if (!sw) {
        if (!haveF) {
          fippi_warp(d, Va, Vb, sgx8, sgw8, N_FIP_ADJ, lane, F);
          haveF = true;
        }
        pair_moments_part<double, true>(g, k, srule6, 6, lane, 32, MG, MP);
        cx_warp_sum(MG, 9);
        cx_warp_sum(MP, 9);
        add_taylor_terms(F, k, MG, MP);
        desing = true;
      } else if (d.ncv == 0) {
        pair_moments_part<double, false>(g, k, c_ho, HO_N * HO_N, lane, 32, MG, MP);
        cx_warp_sum(MG, 9);
        cx_warp_sum(MP, 9);
      } else {
        td_touch(d.ncv, Va, Vb, d.perm_a, d.perm_b, k, c_gx12, c_gw12, N_TD, lane, 32, MG, T);
        cx_warp_sum(MG, 9);
        cx_warp_sum(T, 10);
        for (int q = 0; q < 9; q++) MP[q] = mk(0.0, 0.0);
        td = true;
      }
      VecMoments<double> vm;
      vec_moments(g, MG, MP, &vm);
      vec_combine(g, vm, ja, jb, m4ok2, &H0, &H1);
      if (desing) H1 = H1 + mk(-0.079577471545947667884 * htimes_rm3(F, Va, Vb, ja, jb), 0.0);
      if (td) H1 = td_h1(Va, Vb, T, ja, jb);
    }
    if (lane < 9) {
      const cx<double> v = ra.pf1[r] * (W[0][m] * H0) + ra.pfc[r] * (W[1][m] * H1) + ra.pf3[r] * (W[2][m] * H0);
      E += fac * v.re;
    }
  }
  return warp_sum(E);  // every lane returns the value
}

struct VjpNearArgs {
  VjpTables t;
  const DevNear* near;
  int nnear, bpe_a, bpe_b;
  double rel_step;  // displacement = rel_step * the pair's larger panel radius
};

__global__ void __launch_bounds__(128) vjp_near_kernel(VjpNearArgs a, RegionArgs ra) {
  // 15 warps per pair: vertices 1..5 of the pair's six slots (panel a's
  // vertex 0 follows from the others) x 3 coordinates; each warp evaluates
  // its two displaced pairs with the lanes over the cubature points
  // the rules in shared memory: the lanes read different nodes at once
  __shared__ double sgx[N_FIP_ADJ], sgw[N_FIP_ADJ], srule6[18], srule16[2 * NT_SELF];
  __shared__ cx<double> sW[4][3][9];  // per warp: the pair's weights (kept out of registers)
  if (threadIdx.x < N_FIP_ADJ) { sgx[threadIdx.x] = c_gx8[threadIdx.x]; sgw[threadIdx.x] = c_gw8[threadIdx.x]; }
  if (threadIdx.x < 18) srule6[threadIdx.x] = c_lo64[threadIdx.x];
  if (threadIdx.x < NT_SELF) { srule16[threadIdx.x] = c_gx16[threadIdx.x]; srule16[NT_SELF + threadIdx.x] = c_gw16[threadIdx.x]; }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long pair = wid / 15;
  if (pair >= a.nnear) return;  // whole warps
  const int dir = (int)(wid % 15), v = 1 + dir / 3, c = dir % 3;
  const VjpTables& t = a.t;
  const DevNear d = a.near[pair];
  const bool self = d.pa == d.pb;
  // a pair's value does not change when both panels move together, so the
  // derivative for panel a's vertex 0 is minus the sum of the others': that
  // vertex is not displaced, each other direction subtracts its share from it
  if (v == 0 || (self && v >= 3)) return;
  const int gv = v < 3 ? t.pvi[3 * d.pa + v] : t.pvi[3 * d.pb + v - 3];
  const int g0 = t.pvi[3 * d.pa];
  if (gv == g0) return;
  if (v >= 3)
    for (int q = 0; q < 3; q++)
      if (t.pvi[3 * d.pa + q] == gv) return;  // a shared vertex moves with panel a's slot
  double sgA[3], sgB[3];
  for (int q = 0; q < 3; q++) {
    sgA[q] = t.sbf[3 * d.pa + q] >= 0 ? (t.ssl[3 * d.pa + q] > 0.0 ? 1.0 : -1.0) : 0.0;
    sgB[q] = t.sbf[3 * d.pb + q] >= 0 ? (t.ssl[3 * d.pb + q] > 0.0 ? 1.0 : -1.0) : 0.0;
  }
  cx<double>(*W)[9] = sW[threadIdx.x >> 5];
  if (lane < 9) {
    cx<double> w3[3];
    vjp_weights_m(t, d.pa, d.pb, a.bpe_a, a.bpe_b, !self, lane, w3);
    W[0][lane] = w3[0]; W[1][lane] = w3[1]; W[2][lane] = w3[2];
  }
  __syncwarp();
  const double h = a.rel_step * d.rmax;
  double E[2];
  for (int s = 0; s < 2; s++) {
    double Va[9], Vb[9];
    for (int q = 0; q < 9; q++) { Va[q] = t.pv[9 * (size_t)d.pa + q]; Vb[q] = t.pv[9 * (size_t)d.pb + q]; }
    const double dv = s == 0 ? h : -h;
    for (int q = 0; q < 3; q++) {
      if (t.pvi[3 * d.pa + q] == gv) Va[3 * q + c] += dv;
      if (t.pvi[3 * d.pb + q] == gv) Vb[3 * q + c] += dv;
    }
    E[s] = near_pair_energy(d, Va, Vb, sgA, sgB, ra, W, lane, sgx, sgw, srule6, srule16);
  }
  const double dE = (E[0] - E[1]) / (2.0 * h);
  if (lane == 0) {
    atomicAdd(&t.grad[3 * (size_t)gv + c], dE);
    atomicAdd(&t.grad[3 * (size_t)g0 + c], -dE);
  }
}

struct RhsVjpArgs {
  const double* V;  // surface vertices
  const int* E;     // 8 ints per edge
  const double* elen;
  int ne, bf_offset, pec, sign, voff, nw;
  cx<double> k, Z;
  const double* E0;  // 6 per wave (complex)
  const double* nh;  // 3 per wave
  const cx<double>* gb;
  long long ldg;
  double* grad;
};

// one thread per edge: the gradient of Re sum_w conj(g_iw) b_iw (rhs_kernel's
// integrals) with respect to the edge's four vertices
__global__ void rhs_vjp_kernel(RhsVjpArgs a) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.ne) return;
  const int* ed = a.E + 8 * e;
  const double* V1 = a.V + 3 * ed[0];
  const double* V2 = a.V + 3 * ed[1];
  const double L = a.elen[e];
  const double ZVAC = 376.73031346177;
  const cx<double> ik = mk(-a.k.im, a.k.re);
  double g1[3] = {0.0, 0.0, 0.0}, g2[3] = {0.0, 0.0, 0.0};
  for (int side = 0; side < 2; side++) {
    const int iq = side == 0 ? ed[2] : ed[3];
    if (iq < 0) continue;
    const double ss = side == 0 ? 1.0 : -1.0;
    const double* Q = a.V + 3 * iq;
    double A[3], B[3], gq[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 3; i++) { A[i] = V1[i] - Q[i]; B[i] = V2[i] - Q[i]; }
    double Ire = 0.0;
    for (int w = 0; w < a.nw; w++) {
      const int i0 = a.bf_offset + (a.pec ? e : 2 * e);
      const cx<double> gE = a.gb[i0 + (long long)w * a.ldg];
      const cx<double> gH = a.pec ? mk(0.0, 0.0) : a.gb[i0 + 1 + (long long)w * a.ldg];
      const double* nh = a.nh + 3 * w;
      cx<double> E0[3], P[3];
      for (int i = 0; i < 3; i++) E0[i] = mk(a.E0[6 * w + 2 * i], a.E0[6 * w + 2 * i + 1]);
      // P = (sign/ZVAC) conj(gE) E0 + sign conj(gH) (nh x E0)/Z
      const cx<double> cE = (a.sign / ZVAC) * mk(gE.re, -gE.im);
      const cx<double> cH = cdiv((double)a.sign * mk(gH.re, -gH.im), a.Z);
      cx<double> nxE[3];
      rcvcross(nh, E0, nxE);
      for (int i = 0; i < 3; i++) P[i] = cE * E0[i] + cH * nxE[i];
      for (int q = 0; q < HO_N * HO_N; q++) {
        const double u = c_ho[3 * q], v = c_ho[3 * q + 1], wq = c_ho[3 * q + 2];
        double X[3], F[3];
        for (int i = 0; i < 3; i++) { F[i] = u * A[i] + v * B[i]; X[i] = Q[i] + F[i]; }
        const double ph = nh[0] * X[0] + nh[1] * X[1] + nh[2] * X[2];
        const cx<double> ex = wq * cexpo(mk(-a.k.im * ph, a.k.re * ph));
        const cx<double> FP = F[0] * P[0] + F[1] * P[1] + F[2] * P[2];
        Ire += (FP * ex).re;
        const cx<double> t = FP * ik;
        for (int i = 0; i < 3; i++) {
          const cx<double> dX = (P[i] + nh[i] * t) * ex;  // d(F.P e^{ik nh.X})/dX
          const double dr = ss * L * dX.re;
          g1[i] += u * dr; g2[i] += v * dr;
          gq[i] += (1.0 - u - v) * dr - ss * L * (P[i] * ex).re;
        }
      }
    }
    for (int i = 0; i < 3; i++) {
      const double dl = ss * Ire * (V1[i] - V2[i]) / L;
      g1[i] += dl; g2[i] -= dl;
      atomicAdd(&a.grad[3 * (size_t)(a.voff + iq) + i], gq[i]);
    }
  }
  for (int i = 0; i < 3; i++) {
    atomicAdd(&a.grad[3 * (size_t)(a.voff + ed[0]) + i], g1[i]);
    atomicAdd(&a.grad[3 * (size_t)(a.voff + ed[1]) + i], g2[i]);
  }
}

// per-panel tables of the adjoint (built on first use)
static gbem_status upload_vjp_tables(Geometry* g) {
  if (g->d_pvi) return GBEM_OK;
  const size_t np = (size_t)g->np_total;
  std::vector<int> pvi(3 * np), sbf(3 * np, -1);
  std::vector<double> ssl(3 * np, 0.0);
  int voff = 0;
  for (const Surface& S : g->S) {
    for (int p = 0; p < S.np; p++) {
      const size_t gp = S.panel_offset + p;
      for (int j = 0; j < 3; j++) {
        pvi[3 * gp + j] = voff + S.PV[3 * p + j];
        const int e = S.he_edge[3 * p + j];
        if (e < 0) continue;
        sbf[3 * gp + j] = S.bf_offset + (S.pec ? 1 : 2) * e;
        ssl[3 * gp + j] = (S.he_side[3 * p + j] == 0 ? 1.0 : -1.0) * S.elen[e];
      }
    }
    voff += S.nv;
  }
  cudaError_t e = dupload(&g->d_pvi, pvi.data(), pvi.size());
  if (e == cudaSuccess) e = dupload(&g->d_sbf, sbf.data(), sbf.size());
  if (e == cudaSuccess) e = dupload(&g->d_ssl, ssl.data(), ssl.size());
  return cuda_status(e, "adjoint tables");
}

static int total_vertices(const Geometry* g) {
  int n = 0;
  for (const Surface& S : g->S) n += S.nv;
  return n;
}

gbem_status vertex_vjp_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int nrhs,
                              const void* d_lam, int ldl, const void* d_x, int ldx, double* d_grad, double rel_step,
                              cudaStream_t s, int only_region) {
  gbem_status st = upload_geometry(g);
  if (st == GBEM_OK) st = upload_vjp_tables(g);
  if (st != GBEM_OK) return st;
  VjpTables t;
  t.pv = g->d_pv; t.pc = g->d_pc; t.pvi = g->d_pvi; t.sbf = g->d_sbf; t.ssl = g->d_ssl;
  t.lam = (const cx<double>*)d_lam; t.x = (const cx<double>*)d_x; t.ldl = ldl; t.ldx = ldx; t.nrhs = nrhs;
  t.grad = d_grad;
  cudaError_t e = cudaSuccess;
  for (size_t bi = 0; bi < g->blocks.size() && e == cudaSuccess; bi++) {
    const Block& b = g->blocks[bi];
    const DevBlock* db = g->dblocks[bi];
    if (b.nreg == 0) continue;
    const Surface& A = g->S[b.sa];
    const Surface& B = g->S[b.sb];
    RegionArgs ra = region_args(b, wr, wi, eps, mu);
    if (only_region >= 0) {
      ra = single_region_args(b, ra, only_region, wr, wi, eps, mu);
      if (ra.nreg == 0) continue;
    }
    VjpFarArgs fa;
    fa.t = t; fa.offa = A.panel_offset; fa.offb = B.panel_offset; fa.npa = A.np; fa.npb = B.np;
    fa.bpe_a = A.pec ? 1 : 2; fa.bpe_b = B.pec ? 1 : 2; fa.sym = b.sym ? 1 : 0;
    if (A.np && B.np) {
      vjp_far_kernel<<<dim3((B.np + 127) / 128, A.np), 128, 0, s>>>(fa, ra);
      stats_launch(ST_OTHER);
    }
    if (db->nnear) {
      VjpNearArgs na;
      na.t = t; na.near = db->near; na.nnear = db->nnear; na.bpe_a = fa.bpe_a; na.bpe_b = fa.bpe_b;
      na.rel_step = rel_step;
      const long long n = 15LL * 32 * db->nnear;  // one warp per (pair, displaced coordinate)
      vjp_near_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(na, ra);
      stats_launch(ST_OTHER);
    }
    e = cudaGetLastError();
  }
  return cuda_status(e, "vertex adjoint");
}

gbem_status rhs_vjp_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int nw,
                           const double* E0, const double* nh, const void* d_gb, int ldg, double* d_grad, cudaStream_t s) {
  gbem_status st = upload_geometry(g);
  if (st != GBEM_OK) return st;
  double *dE0 = nullptr, *dnh = nullptr;
  cudaError_t e = dupload(&dE0, E0, 6 * (size_t)nw);
  if (e == cudaSuccess) e = dupload(&dnh, nh, 3 * (size_t)nw);
  int voff = 0;
  for (const Surface& S : g->S) {
    const int vo = voff;
    voff += S.nv;
    if (e != cudaSuccess) break;
    int sign;
    if (S.reg_ext == 0) sign = -1;
    else if (S.reg_int == 0) sign = 1;
    else continue;
    if (!S.ne) continue;
    double *dV = nullptr, *dL = nullptr;
    int* dE = nullptr;
    e = dupload(&dV, S.V.data(), S.V.size());
    if (e == cudaSuccess) e = dupload(&dE, S.E.data(), S.E.size());
    if (e == cudaSuccess) e = dupload(&dL, S.elen.data(), S.elen.size());
    if (e == cudaSuccess) {
      RhsVjpArgs a;
      a.V = dV; a.E = dE; a.elen = dL; a.ne = S.ne; a.bf_offset = S.bf_offset; a.pec = S.pec ? 1 : 0; a.sign = sign;
      a.voff = vo; a.nw = nw;
      cx<double> ep = cxd(eps[0], eps[1]), m = cxd(mu[0], mu[1]), em = ep * m;
      double rr = std::sqrt(std::hypot(em.re, em.im)), th = 0.5 * std::atan2(em.im, em.re);
      a.k = cxd(rr * std::cos(th), rr * std::sin(th)) * cxd(wr, wi);
      cx<double> q = cdiv(m, ep);
      double rq = std::sqrt(std::hypot(q.re, q.im)), tq = 0.5 * std::atan2(q.im, q.re);
      a.Z = 376.73031346177 * cxd(rq * std::cos(tq), rq * std::sin(tq));
      a.E0 = dE0; a.nh = dnh; a.gb = (const cx<double>*)d_gb; a.ldg = ldg; a.grad = d_grad;
      rhs_vjp_kernel<<<(S.ne + 127) / 128, 128, 0, s>>>(a);
      stats_launch(ST_OTHER);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    cudaFree(dV); cudaFree(dE); cudaFree(dL);
  }
  cudaFree(dE0); cudaFree(dnh);
  return cuda_status(e, "rhs adjoint");
}

int geometry_total_vertices(const Geometry* g) { return total_vertices(g); }

}  // namespace gbem
