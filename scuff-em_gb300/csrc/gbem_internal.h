// gbem_internal.h -- host-side data structures shared by the library's
// translation units (never exposed through the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include <cstdint>
#include "../../include/gbem.h"

namespace gbem {

// tile geometry of the far-field assembly: TE edges per side, at most
// PMAX distinct panels per edge block
constexpr int TE = 32;
constexpr int PMAX = 48;

struct Surface {
  int nv = 0, np = 0, ne = 0;
  std::vector<double> V;        // 3 nv
  std::vector<int> PV;          // 3 np
  std::vector<double> cen, rad; // 3 np, np
  std::vector<int> E;           // 8 ne: iV1 iV2 iQP iQM iPPanel iMPanel PIndex MIndex
  std::vector<double> elen;     // ne
  int reg_ext = 0, reg_int = -1;
  bool pec = false;
  int bf_offset = 0;            // first basis-function index in the matrix
  int panel_offset = 0;         // first global panel index
  std::vector<int> he_edge;     // 3 np: edge of (panel, local vertex j) or -1
  std::vector<int> he_side;     // 3 np: 0 = positive panel, 1 = negative panel
};

// a row (or column) block of consecutive edges of one surface
struct EdgeBlock {
  int e0 = 0, ne = 0;                 // edges [e0, e0+ne)
  std::vector<int> panels;            // global panel indices (<= PMAX)
  std::vector<int8_t> he_local;       // 3 per panel: local edge index in block or -1
  std::vector<int8_t> he_side;        // 3 per panel
};

struct NearPair {
  int pa, pb;      // global panel indices (pa <= pb inside a self block)
  int ncv;         // common vertices 0..3
  int8_t perm_a[3], perm_b[3];  // common-vertices-first order -> mesh order
  double rmax;     // larger panel radius
};

// A column stripe of a block for the mixed-precision far field, which runs
// in two passes: every far panel pair of the stripe once (pair values into a
// scratch buffer), then the stripe's edge tiles from those values.
struct Stripe {
  int cb0 = 0, cb1 = 0;     // column edge blocks [cb0, cb1)
  int nrow = 0;             // row panels [0, nrow) (surface-local) the stripe's entries touch
  std::vector<int> cpan;    // column panels (surface-local, ascending) of the stripe's edges
  std::vector<int2> tiles;  // the stripe's tiles (row block, column block)
};

struct Block {
  int sa = 0, sb = 0;
  bool sym = false;
  int nreg = 0;
  int reg[2] = {0, 0};
  double sign[2] = {0, 0};
  int bpe_a = 1, bpe_b = 1;            // basis functions per edge (1 PEC, 2 dielectric)
  std::vector<EdgeBlock> rows, cols;
  std::vector<int2> tiles;             // (row block, col block)
  std::vector<NearPair> near;          // near pairs of this surface pair
  std::vector<int> near_ptr, near_col, near_idx;  // CSR over local row panel: (pb, pair index, transpose flag in sign)
  double rmax_touch = 0.0;             // largest panel radius over the pairs with ncv = 1, 2
  std::vector<Stripe> stripes;         // column stripes (mixed far field)
  std::vector<int2> ecol;              // per column edge: stripe-local index of its P, M panel (-1: none)
  size_t max_stripe_pairs = 0;         // largest nrow * cpan.size() over the stripes
};

struct DevBlock;  // defined in assemble.cu
struct Fippi;     // static near-pair integrals (bem_math.cuh)

struct Geometry {
  int device = 0;
  int nregions = 1;
  int N = 0;
  int np_total = 0;
  std::vector<Surface> S;
  std::vector<Block> blocks;
  long long near_counts[4] = {0, 0, 0, 0};
  // device data (owned)
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;  // the library's stream while a caller's is in use
  double* d_pv = nullptr;    // 9 per global panel
  double* d_pc = nullptr;    // 4 per global panel: centroid, radius
  std::vector<DevBlock*> dblocks;
  bool fippi_ready = false;
  std::string err;
  // matrices created on this geometry keep it alive: destroying the
  // geometry while matrices exist defers the release to the last of them
  int refs = 0;
  bool dead = false;
  float* d_ffnode = nullptr;  // per global panel: 6 rule nodes, float-float offsets from ff_origin (36 floats)
  float* d_ffgeo = nullptr;   // per global panel: V0 - ff_origin, V1 - V0, V2 - V0 as float-float (18 floats)
  void* ppv = nullptr;        // pair-value scratch of the mixed far field
  size_t ppv_bytes = 0;
  // adjoint tables, per global panel (built on first use)
  int* d_pvi = nullptr;       // 3: global vertex indices
  int* d_sbf = nullptr;       // 3: basis function of the edge at each vertex slot, -1 if none
  double* d_ssl = nullptr;    // 3: +-edge length (sign of the panel's side)
  // cached buffers of the mixed-precision solve
  void* mixedM = nullptr;
  void* mixedF = nullptr;
  void* mixed_ws = nullptr;
  int mixed_nrhs = 0;
};

struct Matrix {
  const Geometry* g = nullptr;
  int N = 0, ld = 0, dtype = 0;
  void* d = nullptr;            // device storage
  int* d_ipiv = nullptr;        // device pivots (0-based) after factorisation
  std::vector<int> ipiv;        // host copy (1-based)
  bool factored = false;
  cudaStream_t stream = nullptr;
  void* ws = nullptr;           // LU workspace
  size_t ws_bytes = 0;
};

// geometry.cpp
gbem_status build_geometry(int ns, const gbem_surface_desc* d, int nreg, Geometry* g);
// common-vertex count and common-vertices-first order of a panel pair (AssessPanelPair.cc:52-103)
int assess_pair(const double* Va[3], const double* Vb[3], double rmax, int8_t pa[3], int8_t pb[3]);

// assemble.cu
// block selection: only the (nsa, nsb) surface block, placed at (row0, col0)
struct BlockSel {
  int nsa, nsb, row0, col0;
};
gbem_status assemble_device(Geometry* g, double wr, double wi, const double* eps, const double* mu,
                            int precision, void* dM, int ld, int dtype, cudaStream_t s,
                            const BlockSel* only = nullptr, int only_region = -1);
// gradients dM/dx_mu (out[mu], null to skip) and, for nta rotation axes with
// generators gamma (9 per axis), dM/dtheta (outT[a])
gbem_status assemble_gradient_device(Geometry* g, double wr, double wi, const double* eps, const double* mu,
                                     const BlockSel& sel, void* const out[3], int ld, int dtype, cudaStream_t s,
                                     int nta = 0, const double* gamma = nullptr, void* const* outT = nullptr);
gbem_status upload_geometry(Geometry* g);
void free_geometry_device(Geometry* g);
// adjoint contractions (device arrays, complex128 column-major): grad (3 per
// vertex, surfaces in order) += Re sum conj(lam) dM/dV x, and
// += Re sum conj(gb) db/dV for nw plane waves (E0: 6 doubles, nh: 3 per wave)
// only_region >= 0: that region's contribution alone, with the signs of an
// exterior region (the matrix of the EMT power's quadratic form)
gbem_status vertex_vjp_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int nrhs,
                              const void* d_lam, int ldl, const void* d_x, int ldx, double* d_grad, double rel_step,
                              cudaStream_t s, int only_region = -1);
gbem_status rhs_vjp_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, int nw,
                           const double* E0, const double* nh, const void* d_gb, int ldg, double* d_grad, cudaStream_t s);
int geometry_total_vertices(const Geometry* g);
gbem_status download_fippi(Geometry* g, size_t bi, std::vector<Fippi>& table);

// fippi_cache.cu: the process-wide cache of static near-pair integrals in the
// reference's FIPPI cache format
void cache_register(Geometry* g);
void cache_unregister(Geometry* g);
bool cache_active();
int cache_lookup(const Geometry* g, const Block& b, std::vector<Fippi>& table, std::vector<int>& miss);
void cache_stats(const Geometry* g, long long* hits, long long* misses);

// lu.cu
gbem_status lu_factor_device(void* dA, int N, int ld, int dtype, int* d_ipiv, int* h_info, cudaStream_t s,
                             void** ws, size_t* ws_bytes);
gbem_status lu_solve_device(const void* dA, int N, int ld, int dtype, const int* d_perm, char trans, int nrhs,
                            void* dB, int ldb, void* dY, cudaStream_t s);
// X = A^-1 B for many right-hand sides (blocked: block inverses + GEMM updates)
gbem_status lu_solve_many_device(const void* dA, int N, int ld, int dtype, const int* d_perm, int nrhs, void* dB, int ldb,
                                 cudaStream_t s);
gbem_status residual_device(const void* dA, int lda, int dtype, int N, const double* dX, int ldx, const double* dB,
                            int ldb, int nrhs, double* dR, int ldr, void* part, cudaStream_t s);
// LU solve on a host B whose device workspace is a static array of lu.cu
// (no device allocation); the caller makes the matrix's device current
gbem_status lu_solve_static_scratch(const void* dA, int N, int ld, int dtype, const int* d_perm, char trans, int nrhs,
                                    void* hB, int ldb, cudaStream_t s);
int lu_solve_noalloc_max_n(int dtype);
// column splits of the FP64 residual: its partial-sum workspace holds
// RESID_MAX_SPLIT x 8 x N complex128
constexpr int RESID_MAX_SPLIT = 32;
// the LU tuning tables of the current device, as JSON
std::string lu_tuning_json();

// gemm_tc.cu: keep the calling host thread's LU factorisations off the
// split-BF16 tensor-core updates (exact FP32 SIMT updates instead)
void tc_gemm_thread_off(int off);

// sptrf.cu: symmetric matrices in LAPACK's upper packed storage
// (Bunch-Kaufman A = U D U^T, dsptrf/zsptrf semantics); dtype F64 or C128
gbem_status sp_factor_device(void* dAP, int N, int dtype, int* dipiv, int* h_info, cudaStream_t s);
gbem_status sp_solve_device(const void* dAP, int N, int dtype, const int* dipiv, int nrhs, void* dB, int ldb,
                            cudaStream_t s);
gbem_status sp_pack_device(const void* dA, int lda, int n, int dtype, void* dAP, cudaStream_t s);

// per-stage device timing and launch counts (process-wide; see gbem_stats)
enum Stage { ST_FAR = 0, ST_NEAR = 1, ST_PANEL = 2, ST_GEMM = 3, ST_SOLVE = 4, ST_RESID = 5, ST_OTHER = 6, ST_N = 8 };
void stats_launch(int stage, int n = 1);
struct StatTimer {
  int stage;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  StatTimer(int stage, cudaStream_t s);
  ~StatTimer();
};

// Raise a kernel's dynamic shared-memory limit to what the device allows
// (its opt-in maximum less the kernel's static shared memory), once per
// kernel and device.  The limit is process-wide state of the function:
// setting it to each launch's own size would let concurrent solves of
// different sizes lower it under one another's launches.
cudaError_t allow_max_smem_raw(const void* kernel);
template <typename K> inline cudaError_t allow_max_smem(K* kernel) { return allow_max_smem_raw((const void*)kernel); }

// error helpers
void set_error(const char* fmt, ...);
gbem_status cuda_status(cudaError_t e, const char* what);

// Programmatic dependent launch for the LU's chains of small kernels: a kernel
// launched with launch_pdl may be scheduled while the previous kernel of the
// stream still runs (that kernel's CTAs call pdl_trigger once resident), and
// it calls pdl_wait -- which returns once the previous grid has completed and
// its memory is visible -- before its first access to global memory.  That
// hides the launch latency between dependent kernels.  pdl_wait is a no-op in
// a kernel launched without the attribute.  GBEM_PDL=0 turns the attribute off.
bool pdl_enabled();
// per host thread: whether the current factorisation launches with the
// attribute (set by the LU for its recursive-panel path, where it was
// measured faster; the grid-panel path at N > 16384 ran 5 % slower with it)
void pdl_thread_on(bool on);
#ifdef __CUDACC__
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

}  // namespace gbem
