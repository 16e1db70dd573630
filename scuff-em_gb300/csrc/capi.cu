// capi.cu -- the extern "C" boundary declared in include/gbem.h.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <map>
#include <complex>
#include <mutex>
#include <string>
#include <thread>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

gbem_status cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GBEM_OK;
  set_error("%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GBEM_ENOMEM : GBEM_ECUDA;
}

// ---- stage statistics ----
static std::mutex g_stats_mu;
static bool g_stats_on = false;
static long long g_counts[ST_N] = {0};
struct Pending { int stage; cudaEvent_t a, b; };
static std::vector<Pending> g_pending;
static double g_ms[ST_N] = {0};

void stats_launch(int stage, int n) {
  std::lock_guard<std::mutex> l(g_stats_mu);
  g_counts[stage] += n;
}

StatTimer::StatTimer(int st, cudaStream_t str) : stage(st), s(str) {
  if (!g_stats_on) return;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) { a = b = nullptr; return; }
  cudaEventRecord(a, s);
}
StatTimer::~StatTimer() {
  if (!a) return;
  cudaEventRecord(b, s);
  std::lock_guard<std::mutex> l(g_stats_mu);
  g_pending.push_back({stage, a, b});
}

static void stats_collect() {
  std::lock_guard<std::mutex> l(g_stats_mu);
  for (auto& p : g_pending) {
    float ms = 0;
    cudaEventSynchronize(p.b);
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) g_ms[p.stage] += ms;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  g_pending.clear();
}

gbem_status rhs_planewave_device(Geometry* g, double wr, double wi, const double* eps, const double* mu, const double* E0,
                                 const double* nh, void* d_rhs, cudaStream_t s);

static thread_local bool tl_pdl = false;
void pdl_thread_on(bool on) { tl_pdl = on; }
bool pdl_enabled() {
  static int p = -1;
  if (p < 0) {
    const char* e = getenv("GBEM_PDL");
    p = (e && e[0] == '0') ? 0 : 1;
  }
  return p == 1 && tl_pdl;
}

cudaError_t allow_max_smem_raw(const void* kernel) {
  static std::mutex mu;
  static std::vector<std::pair<int, const void*>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> l(mu);
  for (auto& d : done)
    if (d.first == dev && d.second == kernel) return cudaSuccess;
  int optin = 0;
  cudaFuncAttributes fa;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess) done.emplace_back(dev, kernel);
  return e;
}

static size_t esize(int dtype) { return dtype == GBEM_C128 ? 16 : (dtype == GBEM_C64 ? 8 : 8); }
static bool omega_is_zero(double wr, double wi) { return wr == 0.0 && wi == 0.0; }

static void perm_from_ipiv(const std::vector<int>& ipiv0, std::vector<int>& perm) {
  int N = (int)ipiv0.size();
  perm.resize(N);
  for (int i = 0; i < N; i++) perm[i] = i;
  for (int i = 0; i < N; i++) std::swap(perm[i], perm[ipiv0[i]]);
}

}  // namespace gbem

using namespace gbem;

struct gbem_geometry : public Geometry {};
struct gbem_matrix : public Matrix {
  int* d_perm = nullptr;
};

#define CHECK_CUDA(call, what)                     \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_status(e_, what); \
  } while (0)

// EMT scattered power (EMTPFT.cc:642-700 for the scattered part): with M0 the
// matrix of the exterior region alone (KK = i mu w GC0, KN = NK = -i k GC1,
// NN = -i eps w GC0) and the physical coefficients K and N = -ZVAC * (odd
// entries of the KN vector, RWGGeometry.cc:957-979),
//   P_scat = 1/2 sum_ij [ ZVAC Re(K_i* K_j)(-Re M0_ij) + Re(N_i* N_j) Re(M0_ij)/ZVAC
//                         + Im(K_i* N_j)(-Im M0_ij) + Im(N_i* K_j) Im(M0_ij) ].
// One thread per row, columns in chunks; partial sums per (row block, chunk).
template <typename TM>
static __global__ void emt_quadform(const cx<TM>* M, long long ld, int N, const signed char* type, const cx<double>* X,
                                    long long ldx, int nrhs, int cchunk, double* part) {
  const double ZV = 376.73031346177;
  __shared__ double red[8][128];
  const int i = blockIdx.x * 128 + threadIdx.x;
  const int c0 = blockIdx.y * cchunk, c1 = min(N, c0 + cchunk);
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (i < N) {
    const int ti = type[i];
    for (int j = c0; j < c1; j++) {
      const cx<TM> m = M[i + (long long)j * ld];
      const double mr = (double)m.re, mi = (double)m.im;
      const int tj = type[j];
      for (int r = 0; r < nrhs; r++) {
        cx<double> ci = X[i + (long long)r * ldx], cj = X[j + (long long)r * ldx];
        if (ti) ci = (-ZV) * ci;
        if (tj) cj = (-ZV) * cj;
        const double re = ci.re * cj.re + ci.im * cj.im, im = ci.re * cj.im - ci.im * cj.re;  // conj(ci) cj
        double t;
        if (!ti && !tj) t = -ZV * re * mr;
        else if (ti && tj) t = re * mr / ZV;
        else if (!ti) t = -im * mi;
        else t = im * mi;
        acc[r] += t;
      }
    }
  }
  for (int r = 0; r < nrhs; r++) {
    red[r][threadIdx.x] = acc[r];
  }
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int r = 0; r < nrhs; r++) red[r][threadIdx.x] += red[r][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int r = 0; r < nrhs; r++) part[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 8 + r] = red[r][0];
}

// Gradient of the EMT scattered power with respect to the solution vector:
// P = 1/2 c^H H c with c = D x (D = 1 on K rows, -ZVAC on N rows) and
// H = S - i T, S_ij = alpha_ij Re M0_ij (alpha: KK -ZVAC, NN 1/ZVAC),
// T_ij = beta_ij Im M0_ij (beta: KN -1, NK +1), the form of emt_quadform;
// out = dP/dRe x + i dP/dIm x = D H D x.  One thread per row.
static __global__ void emt_grad(const cx<double>* M, long long ld, int N, const signed char* type, const cx<double>* X,
                                long long ldx, int nrhs, cx<double>* out, long long ldo) {
  const double ZV = 376.73031346177;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int ti = type[i];
  double gr[8] = {0, 0, 0, 0, 0, 0, 0, 0}, gi[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < N; j++) {
    const cx<double> m = M[i + (long long)j * ld];
    const int tj = type[j];
    const double s = (!ti && !tj) ? -ZV * m.re : ((ti && tj) ? m.re / ZV : 0.0);
    const double t = (!ti && tj) ? -m.im : ((ti && !tj) ? m.im : 0.0);
    const double dj = tj ? -ZV : 1.0;
    for (int r = 0; r < nrhs; r++) {
      const cx<double> xj = X[j + (long long)r * ldx];
      const double cr = dj * xj.re, ci = dj * xj.im;
      // (s - i t) (cr + i ci)
      gr[r] += s * cr + t * ci;
      gi[r] += s * ci - t * cr;
    }
  }
  const double di = ti ? -ZV : 1.0;
  for (int r = 0; r < nrhs; r++) out[i + (long long)r * ldo] = mk(di * gr[r], di * gi[r]);
}

namespace gbem {
template <typename T>
static __global__ void trace_diag(const cx<T>* X, long long ldx, int n, double* out) {
  __shared__ double sr[1024], si[1024];
  double ar = 0.0, ai = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cx<T> v = X[i + (long long)i * ldx];
    ar += (double)v.re;
    ai += (double)v.im;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) { sr[threadIdx.x] += sr[threadIdx.x + o]; si[threadIdx.x] += si[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = sr[0]; out[1] = si[0]; }
}

// sum of log|U(n,n)| over the diagonal of an LU factor; complex entries by
// their modulus
template <typename T>
static __global__ void log_abs_diag(const T* A, long long ld, int n, int cplx, double* out) {
  __shared__ double sr[1024];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const long long o = (long long)i * (ld + 1);
    double m;
    if (cplx) m = hypot((double)A[2 * o], (double)A[2 * o + 1]);
    else m = fabs((double)A[o]);
    acc += log(m);
  }
  sr[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sr[threadIdx.x] += sr[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = sr[0];
}

}  // namespace gbem

extern "C" {

const char* gbem_last_error(void) { return g_err; }
const char* gbem_version(void) { return "gbem 0.1 (sm_103a)"; }

gbem_status gbem_geometry_create(int num_surfaces, const gbem_surface_desc* surfaces, int num_regions, int device,
                                 gbem_geometry** out) {
  if (!out) { set_error("gbem_geometry_create: out is NULL"); return GBEM_EINVAL; }
  *out = nullptr;
  gbem_geometry* g = new (std::nothrow) gbem_geometry();
  if (!g) { set_error("out of host memory"); return GBEM_ENOMEM; }
  g->device = device;
  gbem_status st = build_geometry(num_surfaces, surfaces, num_regions, g);
  if (st != GBEM_OK) { delete g; return st; }
  // no CUDA call here: the device stream is created on first device use, so
  // the mesh bookkeeping also works on a host without a GPU
  cache_register(g);
  *out = g;
  return GBEM_OK;
}

static gbem_status ensure_stream(gbem_geometry* g) {
  cudaError_t e = cudaSetDevice(g->device);
  if (e == cudaSuccess && !g->stream) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  return cuda_status(e, "device setup");
}

static void geometry_release(gbem_geometry* g) {
  cache_unregister(g);
  if (g->stream) {
    cudaSetDevice(g->device);
    cudaStreamSynchronize(g->stream);
  }
  cudaFree(g->mixed_ws);
  g->mixed_ws = nullptr;
  if (g->d_pv) free_geometry_device(g);
  if (g->own_stream) cudaStreamDestroy(g->own_stream);
  else if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

gbem_status gbem_geometry_destroy(gbem_geometry* g) {
  if (!g) return GBEM_OK;
  if (g->mixedM) {
    gbem_matrix* a = (gbem_matrix*)g->mixedM;
    gbem_matrix* b = (gbem_matrix*)g->mixedF;
    g->mixedM = g->mixedF = nullptr;
    gbem_matrix_destroy(a);
    gbem_matrix_destroy(b);
  }
  if (g->refs > 0) {  // live matrices still use the geometry's stream
    g->dead = true;
    return GBEM_OK;
  }
  geometry_release(g);
  return GBEM_OK;
}

gbem_status gbem_geometry_set_stream(gbem_geometry* g, void* stream) {
  if (!g) { set_error("gbem_geometry_set_stream: NULL geometry"); return GBEM_EINVAL; }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  if (!g->own_stream) g->own_stream = g->stream;
  cudaStreamSynchronize(g->stream);
  g->stream = stream ? (cudaStream_t)stream : g->own_stream;
  if (g->mixedM) { ((gbem_matrix*)g->mixedM)->stream = g->stream; ((gbem_matrix*)g->mixedF)->stream = g->stream; }
  return GBEM_OK;
}

gbem_status gbem_geometry_num_bfs(const gbem_geometry* g, int* N) {
  if (!g || !N) { set_error("gbem_geometry_num_bfs: NULL argument"); return GBEM_EINVAL; }
  *N = g->N;
  return GBEM_OK;
}

gbem_status gbem_geometry_edges(const gbem_geometry* g, int surface, int* num_edges, int* edge_table, double* lengths) {
  if (!g || surface < 0 || surface >= (int)g->S.size() || !num_edges) {
    set_error("gbem_geometry_edges: bad arguments");
    return GBEM_EINVAL;
  }
  const Surface& s = g->S[surface];
  *num_edges = s.ne;
  if (edge_table) memcpy(edge_table, s.E.data(), sizeof(int) * s.E.size());
  if (lengths) memcpy(lengths, s.elen.data(), sizeof(double) * s.elen.size());
  return GBEM_OK;
}

gbem_status gbem_geometry_near_counts(const gbem_geometry* g, long long counts[4]) {
  if (!g || !counts) { set_error("gbem_geometry_near_counts: NULL argument"); return GBEM_EINVAL; }
  for (int i = 0; i < 4; i++) counts[i] = g->near_counts[i];
  return GBEM_OK;
}

gbem_status gbem_matrix_create(const gbem_geometry* g, int dtype, gbem_matrix** out) {
  if (!g || !out || (dtype != GBEM_C128 && dtype != GBEM_C64 && dtype != GBEM_F64)) {
    set_error("gbem_matrix_create: bad arguments (dtype must be C128, C64 or F64)");
    return GBEM_EINVAL;
  }
  *out = nullptr;
  gbem_status st0 = ensure_stream(const_cast<gbem_geometry*>(g));
  if (st0 != GBEM_OK) return st0;
  gbem_matrix* m = new gbem_matrix();
  m->g = g; m->N = g->N; m->ld = g->N; m->dtype = dtype; m->stream = g->stream;
  cudaError_t e = cudaMalloc(&m->d, (size_t)m->N * m->ld * esize(dtype));
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_ipiv, sizeof(int) * m->N);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->d_perm, sizeof(int) * m->N);
  if (e != cudaSuccess) {
    cudaFree(m->d); cudaFree(m->d_ipiv); cudaFree(m->d_perm);
    delete m;
    return cuda_status(e, "gbem_matrix_create");
  }
  const_cast<gbem_geometry*>(g)->refs++;
  *out = m;
  return GBEM_OK;
}

gbem_status gbem_matrix_destroy(gbem_matrix* m) {
  if (!m) return GBEM_OK;
  cudaStreamSynchronize(m->stream);
  cudaFree(m->d); cudaFree(m->d_ipiv); cudaFree(m->d_perm); cudaFree(m->ws);
  gbem_geometry* g = const_cast<gbem_geometry*>(static_cast<const gbem_geometry*>(m->g));
  delete m;
  if (g && --g->refs == 0 && g->dead) geometry_release(g);
  return GBEM_OK;
}

gbem_status gbem_matrix_device_ptr(gbem_matrix* m, void** dptr, int* ld) {
  if (!m || !dptr) { set_error("gbem_matrix_device_ptr: NULL argument"); return GBEM_EINVAL; }
  *dptr = m->d;
  if (ld) *ld = m->ld;
  return GBEM_OK;
}

gbem_status gbem_matrix_download(gbem_matrix* m, void* host, int ldh) {
  if (!m || !host || ldh < m->N) { set_error("gbem_matrix_download: bad arguments"); return GBEM_EINVAL; }
  size_t es = esize(m->dtype);
  CHECK_CUDA(cudaMemcpy2DAsync(host, (size_t)ldh * es, m->d, (size_t)m->ld * es, (size_t)m->N * es, m->N,
                               cudaMemcpyDeviceToHost, m->stream), "download");
  CHECK_CUDA(cudaStreamSynchronize(m->stream), "download");
  return GBEM_OK;
}

gbem_status gbem_matrix_upload(gbem_matrix* m, const void* host, int ldh) {
  if (!m || !host || ldh < m->N) { set_error("gbem_matrix_upload: bad arguments"); return GBEM_EINVAL; }
  size_t es = esize(m->dtype);
  CHECK_CUDA(cudaMemcpy2DAsync(m->d, (size_t)m->ld * es, host, (size_t)ldh * es, (size_t)m->N * es, m->N,
                               cudaMemcpyHostToDevice, m->stream), "upload");
  CHECK_CUDA(cudaStreamSynchronize(m->stream), "upload");
  m->factored = false;
  return GBEM_OK;
}

// real parts of an m x n complex128 block (the reference's real storage at
// imaginary frequency, where the matrix is real)
static __global__ void take_real(const double2* src, long long lds, double* dst, long long ldd, int m, int n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)m * n) return;
  const int i = (int)(t % m), j = (int)(t / m);
  dst[i + j * ldd] = src[i + j * lds].x;
}
static __global__ void make_complex(const double* src, long long lds, double2* dst, long long ldd, int m, int n) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)m * n) return;
  const int i = (int)(t % m), j = (int)(t / m);
  dst[i + j * ldd] = make_double2(src[i + j * lds], 0.0);
}

static int surface_bfs(const gbem_geometry* g, int ns) { return g->S[ns].ne * (g->S[ns].pec ? 1 : 2); }

// assembly of the whole matrix (sel = NULL) or of one surface block into a
// device array; F64 goes through a complex128 block whose real part is kept
static gbem_status assemble_into(gbem_geometry* g, double wr, double wi, const double* eps, const double* mu,
                                 int precision, void* dst, int ld, int dtype, const BlockSel* sel) {
  if (omega_is_zero(wr, wi)) { set_error("gbem_assemble: Omega = 0 is not supported"); return GBEM_EINVAL; }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  cudaStream_t s = g->stream;
  if (dtype != GBEM_F64) return assemble_device(g, wr, wi, eps, mu, precision, dst, ld, dtype, s, sel);
  if (precision != GBEM_PREC_FP64) { set_error("gbem_assemble: F64 storage needs the FP64 precision"); return GBEM_EINVAL; }
  const int m = sel ? surface_bfs(g, sel->nsa) : g->N, n = sel ? surface_bfs(g, sel->nsb) : g->N;
  void* tmp = nullptr;
  CHECK_CUDA(cudaMallocAsync(&tmp, (size_t)m * n * 16, s), "F64 assembly scratch");
  BlockSel local;
  if (sel) { local = *sel; local.row0 = 0; local.col0 = 0; }
  st = assemble_device(g, wr, wi, eps, mu, GBEM_PREC_FP64, tmp, m, GBEM_C128, s, sel ? &local : nullptr);
  if (st == GBEM_OK) {
    double* d = (double*)dst + (sel ? (size_t)sel->row0 + (size_t)sel->col0 * ld : 0);
    take_real<<<(unsigned)(((long long)m * n + 255) / 256), 256, 0, s>>>((const double2*)tmp, m, d, ld, m, n);
    stats_launch(ST_OTHER);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_status(e, "take_real");
  }
  cudaFreeAsync(tmp, s);
  return st;
}

gbem_status gbem_assemble(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                          int precision, gbem_matrix* M) {
  if (!g || !M || !eps || !mu || M->N != g->N) { set_error("gbem_assemble: bad arguments"); return GBEM_EINVAL; }
  M->factored = false;
  return assemble_into(g, omega_re, omega_im, eps, mu, precision, M->d, M->ld, M->dtype, nullptr);
}

gbem_status gbem_assemble_block(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                const double* eps, const double* mu, int precision, void* dst, int ld, int row0,
                                int col0, int dtype) {
  if (!g || !dst || !eps || !mu || nsa < 0 || nsb < 0 || nsa >= (int)g->S.size() || nsb >= (int)g->S.size() ||
      row0 < 0 || col0 < 0 || ld < row0 + surface_bfs(g, nsa) ||
      (dtype != GBEM_C128 && dtype != GBEM_C64 && dtype != GBEM_F64)) {
    set_error("gbem_assemble_block: bad arguments");
    return GBEM_EINVAL;
  }
  BlockSel sel{nsa, nsb, row0, col0};
  return assemble_into(g, omega_re, omega_im, eps, mu, precision, dst, ld, dtype, &sel);
}

gbem_status gbem_power_emt(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                           int precision, int nrhs, const double* KN, int ldkn, const double* rhs, int ldr,
                           double* pscat, double* pext) {
  if (!g || !eps || !mu || !KN || !pscat || nrhs <= 0 || nrhs > 8 || ldkn < g->N || (rhs && ldr < g->N)) {
    set_error("gbem_power_emt: bad arguments (1 <= nrhs <= 8)");
    return GBEM_EINVAL;
  }
  for (const Surface& S : g->S)
    if (S.reg_ext != 0) {
      set_error("gbem_power_emt: every surface must face the exterior region 0 (nested bodies are not supported)");
      return GBEM_ENOTSUP;
    }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  const int N = g->N;
  cudaStream_t s = g->stream;
  const int dtype = precision == GBEM_PREC_MIXED ? GBEM_C64 : GBEM_C128;
  std::vector<signed char> type(N);
  for (const Surface& S : g->S)
    for (int e = 0; e < S.ne; e++) {
      if (S.pec) type[S.bf_offset + e] = 0;
      else { type[S.bf_offset + 2 * e] = 0; type[S.bf_offset + 2 * e + 1] = 1; }
    }
  const int nsplit = 8, cchunk = (N + nsplit - 1) / nsplit, nb = (N + 127) / 128;
  void *dM = nullptr, *dX = nullptr, *dT = nullptr, *dP = nullptr;
  cudaError_t e = cudaMallocAsync(&dM, (size_t)N * N * (dtype == GBEM_C64 ? 8 : 16), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dX, (size_t)N * nrhs * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dT, (size_t)N, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dP, sizeof(double) * 8 * nb * nsplit, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dX, (size_t)N * 16, KN, (size_t)ldkn * 16, (size_t)N * 16, nrhs, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dT, type.data(), N, cudaMemcpyHostToDevice, s);
  st = cuda_status(e, "gbem_power_emt setup");
  if (st == GBEM_OK) st = assemble_device(g, omega_re, omega_im, eps, mu, precision, dM, N, dtype, s, nullptr, 0);
  std::vector<double> part((size_t)8 * nb * nsplit);
  if (st == GBEM_OK) {
    dim3 grid(nb, nsplit);
    if (dtype == GBEM_C64)
      emt_quadform<float><<<grid, 128, 0, s>>>((const cx<float>*)dM, N, N, (const signed char*)dT, (const cx<double>*)dX,
                                                N, nrhs, cchunk, (double*)dP);
    else
      emt_quadform<double><<<grid, 128, 0, s>>>((const cx<double>*)dM, N, N, (const signed char*)dT,
                                                 (const cx<double>*)dX, N, nrhs, cchunk, (double*)dP);
    stats_launch(ST_OTHER);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), dP, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e, "gbem_power_emt");
  }
  cudaFreeAsync(dM, s); cudaFreeAsync(dX, s); cudaFreeAsync(dT, s); cudaFreeAsync(dP, s);
  cudaStreamSynchronize(s);
  if (st != GBEM_OK) return st;
  const double ZV = 376.73031346177;
  for (int r = 0; r < nrhs; r++) {
    double sum = 0.0;
    for (int b = 0; b < nb * nsplit; b++) sum += part[(size_t)b * 8 + r];
    pscat[r] = 0.5 * sum;
    if (pext && rhs) {
      // extinction: -1/2 ZVAC sum Re(conj(x_i) b_i), with the opposite sign on N rows
      double ext = 0.0;
      for (int i = 0; i < N; i++) {
        const double* x = KN + 2 * ((size_t)i + (size_t)r * ldkn);
        const double* b = rhs + 2 * ((size_t)i + (size_t)r * ldr);
        const double v = x[0] * b[0] + x[1] * b[1];
        ext += type[i] ? -v : v;
      }
      pext[r] = -0.5 * ZV * ext;
    }
  }
  return GBEM_OK;
}

static gbem_status vertex_vjp_impl(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                   const double* mu, int region, int nrhs, const double* lam, int ldl, const double* x,
                                   int ldx, double rel_step, double* grad);

gbem_status gbem_vertex_vjp_matrix(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                   const double* mu, int nrhs, const double* lam, int ldl, const double* x, int ldx,
                                   double rel_step, double* grad) {
  return vertex_vjp_impl(g, omega_re, omega_im, eps, mu, -1, nrhs, lam, ldl, x, ldx, rel_step, grad);
}

gbem_status gbem_vertex_vjp_region(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                   const double* mu, int region, int nrhs, const double* lam, int ldl, const double* x,
                                   int ldx, double rel_step, double* grad) {
  if (!g || region < 0 || region >= g->nregions) {
    set_error("gbem_vertex_vjp_region: region out of range");
    return GBEM_EINVAL;
  }
  return vertex_vjp_impl(g, omega_re, omega_im, eps, mu, region, nrhs, lam, ldl, x, ldx, rel_step, grad);
}

static gbem_status vertex_vjp_impl(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                   const double* mu, int region, int nrhs, const double* lam, int ldl, const double* x,
                                   int ldx, double rel_step, double* grad) {
  if (!g || !eps || !mu || !lam || !x || !grad || nrhs <= 0 || ldl < g->N || ldx < g->N || !(rel_step > 0.0)) {
    set_error("gbem_vertex_vjp_matrix: bad arguments");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  cudaStream_t s = g->stream;
  const int N = g->N, nv = geometry_total_vertices(g);
  void *dL = nullptr, *dX = nullptr, *dG = nullptr;
  cudaError_t e = cudaMallocAsync(&dL, (size_t)N * nrhs * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dX, (size_t)N * nrhs * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dG, sizeof(double) * 3 * (size_t)std::max(nv, 1), s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dL, (size_t)N * 16, lam, (size_t)ldl * 16, (size_t)N * 16, nrhs, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dX, (size_t)N * 16, x, (size_t)ldx * 16, (size_t)N * 16, nrhs, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dG, 0, sizeof(double) * 3 * (size_t)nv, s);
  st = cuda_status(e, "gbem_vertex_vjp_matrix setup");
  if (st == GBEM_OK)
    st = vertex_vjp_device(g, omega_re, omega_im, eps, mu, nrhs, dL, N, dX, N, (double*)dG, rel_step, s, region);
  if (st == GBEM_OK) {
    e = cudaMemcpyAsync(grad, dG, sizeof(double) * 3 * (size_t)nv, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e, "gbem_vertex_vjp_matrix");
  }
  cudaFreeAsync(dL, s); cudaFreeAsync(dX, s); cudaFreeAsync(dG, s);
  cudaStreamSynchronize(s);
  return st;
}

gbem_status gbem_power_emt_grad(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                                int nrhs, const double* KN, int ldkn, double* G, int ldg) {
  if (!g || !eps || !mu || !KN || !G || nrhs <= 0 || nrhs > 8 || ldkn < g->N || ldg < g->N) {
    set_error("gbem_power_emt_grad: bad arguments (1 <= nrhs <= 8)");
    return GBEM_EINVAL;
  }
  for (const Surface& S : g->S)
    if (S.reg_ext != 0) {
      set_error("gbem_power_emt_grad: every surface must face the exterior region 0");
      return GBEM_ENOTSUP;
    }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  const int N = g->N;
  cudaStream_t s = g->stream;
  std::vector<signed char> type(N);
  for (const Surface& S : g->S)
    for (int e = 0; e < S.ne; e++) {
      if (S.pec) type[S.bf_offset + e] = 0;
      else { type[S.bf_offset + 2 * e] = 0; type[S.bf_offset + 2 * e + 1] = 1; }
    }
  void *dM = nullptr, *dX = nullptr, *dT = nullptr, *dG = nullptr;
  cudaError_t e = cudaMallocAsync(&dM, (size_t)N * N * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dX, (size_t)N * nrhs * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dG, (size_t)N * nrhs * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dT, (size_t)N, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dX, (size_t)N * 16, KN, (size_t)ldkn * 16, (size_t)N * 16, nrhs, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dT, type.data(), N, cudaMemcpyHostToDevice, s);
  st = cuda_status(e, "gbem_power_emt_grad setup");
  if (st == GBEM_OK) st = assemble_device(g, omega_re, omega_im, eps, mu, GBEM_PREC_FP64, dM, N, GBEM_C128, s, nullptr, 0);
  if (st == GBEM_OK) {
    emt_grad<<<(N + 127) / 128, 128, 0, s>>>((const cx<double>*)dM, N, N, (const signed char*)dT,
                                            (const cx<double>*)dX, N, nrhs, (cx<double>*)dG, N);
    stats_launch(ST_OTHER);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(G, (size_t)ldg * 16, dG, (size_t)N * 16, (size_t)N * 16, nrhs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e, "gbem_power_emt_grad");
  }
  cudaFreeAsync(dM, s); cudaFreeAsync(dX, s); cudaFreeAsync(dT, s); cudaFreeAsync(dG, s);
  cudaStreamSynchronize(s);
  return st;
}

gbem_status gbem_vertex_vjp_rhs_planewave(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                          const double* mu, int nwaves, const double* E0, const double* nhat,
                                          const double* gb, int ldg, double* grad) {
  if (!g || !eps || !mu || !E0 || !nhat || !gb || !grad || nwaves <= 0 || ldg < g->N) {
    set_error("gbem_vertex_vjp_rhs_planewave: bad arguments");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  cudaStream_t s = g->stream;
  const int N = g->N, nv = geometry_total_vertices(g);
  void *dB = nullptr, *dG = nullptr;
  cudaError_t e = cudaMallocAsync(&dB, (size_t)N * nwaves * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dG, sizeof(double) * 3 * (size_t)std::max(nv, 1), s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dB, (size_t)N * 16, gb, (size_t)ldg * 16, (size_t)N * 16, nwaves, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dG, 0, sizeof(double) * 3 * (size_t)nv, s);
  st = cuda_status(e, "gbem_vertex_vjp_rhs_planewave setup");
  if (st == GBEM_OK) st = rhs_vjp_device(g, omega_re, omega_im, eps, mu, nwaves, E0, nhat, dB, N, (double*)dG, s);
  if (st == GBEM_OK) {
    e = cudaMemcpyAsync(grad, dG, sizeof(double) * 3 * (size_t)nv, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    st = cuda_status(e, "gbem_vertex_vjp_rhs_planewave");
  }
  cudaFreeAsync(dB, s); cudaFreeAsync(dG, s);
  cudaStreamSynchronize(s);
  return st;
}

gbem_status gbem_cache_lookup_stats(const gbem_geometry* g, long long* hits, long long* misses) {
  if (!g || !hits || !misses) { set_error("gbem_cache_lookup_stats: NULL argument"); return GBEM_EINVAL; }
  cache_stats(g, hits, misses);
  return GBEM_OK;
}

gbem_status gbem_geometry_num_vertices(const gbem_geometry* g, int* nv) {
  if (!g || !nv) { set_error("gbem_geometry_num_vertices: NULL argument"); return GBEM_EINVAL; }
  *nv = geometry_total_vertices(g);
  return GBEM_OK;
}

gbem_status gbem_assemble_block_gradient(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                         const double* eps, const double* mu, void* gx, void* gy, void* gz, int ld,
                                         int row0, int col0, int dtype) {
  if (!g || !eps || !mu || nsa < 0 || nsb < 0 || nsa >= (int)g->S.size() || nsb >= (int)g->S.size() || row0 < 0 ||
      col0 < 0 || ld < row0 + surface_bfs(g, nsa) || (dtype != GBEM_C128 && dtype != GBEM_F64)) {
    set_error("gbem_assemble_block_gradient: bad arguments (dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  if (omega_is_zero(omega_re, omega_im)) { set_error("gbem_assemble_block_gradient: Omega = 0"); return GBEM_EINVAL; }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  void* const out[3] = {gx, gy, gz};
  BlockSel sel{nsa, nsb, row0, col0};
  return assemble_gradient_device(g, omega_re, omega_im, eps, mu, sel, out, ld, dtype, g->stream);
}

gbem_status gbem_assemble_block_gradient_host(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                              const double* eps, const double* mu, void* gx, void* gy, void* gz,
                                              int ld, int row0, int col0, int dtype) {
  if (!g || nsa < 0 || nsb < 0 || nsa >= (int)g->S.size() || nsb >= (int)g->S.size() ||
      (dtype != GBEM_C128 && dtype != GBEM_F64) || row0 < 0 || col0 < 0 || ld < row0 + surface_bfs(g, nsa)) {
    set_error("gbem_assemble_block_gradient_host: bad arguments (dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  const int m = surface_bfs(g, nsa), n = surface_bfs(g, nsb);
  const size_t es = dtype == GBEM_C128 ? 16 : 8;
  void* host[3] = {gx, gy, gz};
  void* d[3] = {nullptr, nullptr, nullptr};
  for (int c = 0; c < 3; c++)
    if (host[c]) CHECK_CUDA(cudaMallocAsync(&d[c], (size_t)m * n * es, g->stream), "gradient scratch");
  st = gbem_assemble_block_gradient(g, nsa, nsb, omega_re, omega_im, eps, mu, d[0], d[1], d[2], m, 0, 0, dtype);
  for (int c = 0; c < 3 && st == GBEM_OK; c++) {
    if (!host[c]) continue;
    cudaError_t e = cudaMemcpy2DAsync((char*)host[c] + ((size_t)row0 + (size_t)col0 * ld) * es, (size_t)ld * es, d[c],
                                      (size_t)m * es, (size_t)m * es, n, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) st = cuda_status(e, "gradient download");
  }
  for (int c = 0; c < 3; c++) cudaFreeAsync(d[c], g->stream);
  cudaStreamSynchronize(g->stream);
  return st;
}

gbem_status gbem_assemble_block_dmdt(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                     const double* eps, const double* mu, int naxes, const double* gamma,
                                     void* const* out, int ld, int row0, int col0, int dtype) {
  if (!g || !eps || !mu || !gamma || !out || naxes < 1 || naxes > 3 || nsa < 0 || nsb < 0 ||
      nsa >= (int)g->S.size() || nsb >= (int)g->S.size() || row0 < 0 || col0 < 0 || ld < row0 + surface_bfs(g, nsa) ||
      (dtype != GBEM_C128 && dtype != GBEM_F64)) {
    set_error("gbem_assemble_block_dmdt: bad arguments (1 <= naxes <= 3, dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  if (omega_is_zero(omega_re, omega_im)) { set_error("gbem_assemble_block_dmdt: Omega = 0"); return GBEM_EINVAL; }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  void* const none[3] = {nullptr, nullptr, nullptr};
  BlockSel sel{nsa, nsb, row0, col0};
  return assemble_gradient_device(g, omega_re, omega_im, eps, mu, sel, none, ld, dtype, g->stream, naxes, gamma, out);
}

gbem_status gbem_assemble_block_dmdt_host(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                          const double* eps, const double* mu, int naxes, const double* gamma,
                                          void* const* out, int ld, int row0, int col0, int dtype) {
  if (!g || !out || naxes < 1 || naxes > 3 || nsa < 0 || nsb < 0 || nsa >= (int)g->S.size() ||
      nsb >= (int)g->S.size() || (dtype != GBEM_C128 && dtype != GBEM_F64) || row0 < 0 || col0 < 0 ||
      ld < row0 + surface_bfs(g, nsa)) {
    set_error("gbem_assemble_block_dmdt_host: bad arguments (1 <= naxes <= 3, dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  const int m = surface_bfs(g, nsa), n = surface_bfs(g, nsb);
  const size_t es = dtype == GBEM_C128 ? 16 : 8;
  void* d[3] = {nullptr, nullptr, nullptr};
  for (int c = 0; c < naxes; c++) {
    if (!out[c]) { set_error("gbem_assemble_block_dmdt_host: NULL output"); st = GBEM_EINVAL; break; }
    cudaError_t e = cudaMallocAsync(&d[c], (size_t)m * n * es, g->stream);
    if (e != cudaSuccess) { st = cuda_status(e, "dMdT scratch"); break; }
  }
  if (st == GBEM_OK) st = gbem_assemble_block_dmdt(g, nsa, nsb, omega_re, omega_im, eps, mu, naxes, gamma, d, m, 0, 0, dtype);
  for (int c = 0; c < naxes && st == GBEM_OK; c++) {
    cudaError_t e = cudaMemcpy2DAsync((char*)out[c] + ((size_t)row0 + (size_t)col0 * ld) * es, (size_t)ld * es, d[c],
                                      (size_t)m * es, (size_t)m * es, n, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) st = cuda_status(e, "dMdT download");
  }
  for (int c = 0; c < 3; c++)
    if (d[c]) cudaFreeAsync(d[c], g->stream);
  cudaStreamSynchronize(g->stream);
  return st;
}

gbem_status gbem_assemble_block_host(gbem_geometry* g, int nsa, int nsb, double omega_re, double omega_im,
                                     const double* eps, const double* mu, void* host, int ld, int row0, int col0,
                                     int dtype) {
  if (!g || !host || nsa < 0 || nsb < 0 || nsa >= (int)g->S.size() || nsb >= (int)g->S.size() ||
      (dtype != GBEM_C128 && dtype != GBEM_F64) || row0 < 0 || col0 < 0 || ld < row0 + surface_bfs(g, nsa)) {
    set_error("gbem_assemble_block_host: bad arguments (dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  const int m = surface_bfs(g, nsa), n = surface_bfs(g, nsb);
  const size_t es = dtype == GBEM_C128 ? 16 : 8;
  void* d = nullptr;
  CHECK_CUDA(cudaMallocAsync(&d, (size_t)m * n * es, g->stream), "block scratch");
  st = gbem_assemble_block(g, nsa, nsb, omega_re, omega_im, eps, mu, GBEM_PREC_FP64, d, m, 0, 0, dtype);
  if (st == GBEM_OK) {
    cudaError_t e = cudaMemcpy2DAsync((char*)host + ((size_t)row0 + (size_t)col0 * ld) * es, (size_t)ld * es, d,
                                      (size_t)m * es, (size_t)m * es, n, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) st = cuda_status(e, "block download");
  }
  cudaFreeAsync(d, g->stream);
  cudaStreamSynchronize(g->stream);
  return st;
}

gbem_status gbem_assemble_host(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                               double* ZM, int ld) {
  if (!g || !ZM || ld < g->N) { set_error("gbem_assemble_host: bad arguments"); return GBEM_EINVAL; }
  gbem_matrix* M = nullptr;
  gbem_status st = gbem_matrix_create(g, GBEM_C128, &M);
  if (st != GBEM_OK) return st;
  st = gbem_assemble(g, omega_re, omega_im, eps, mu, GBEM_PREC_FP64, M);
  if (st == GBEM_OK) st = gbem_matrix_download(M, ZM, ld);
  gbem_matrix_destroy(M);
  return st;
}

gbem_status gbem_lu_factor(gbem_matrix* M, int* ipiv, int* info) {
  if (!M) { set_error("gbem_lu_factor: NULL matrix"); return GBEM_EINVAL; }
  CHECK_CUDA(cudaSetDevice(M->g->device), "cudaSetDevice");
  int h_info = 0;
  gbem_status st;
  if (M->dtype == GBEM_F64) {
    // real matrix (dgetrf semantics): factored as complex128 with zero
    // imaginary parts, which stay exactly zero; |Re|+|Im| is then IDAMAX's |x|
    const int N = M->N;
    void* tmp = nullptr;
    CHECK_CUDA(cudaMallocAsync(&tmp, (size_t)N * N * 16, M->stream), "F64 LU scratch");
    const unsigned nb = (unsigned)(((long long)N * N + 255) / 256);
    make_complex<<<nb, 256, 0, M->stream>>>((const double*)M->d, M->ld, (double2*)tmp, N, N, N);
    st = lu_factor_device(tmp, N, N, GBEM_C128, M->d_ipiv, &h_info, M->stream, &M->ws, &M->ws_bytes);
    if (st == GBEM_OK) take_real<<<nb, 256, 0, M->stream>>>((const double2*)tmp, N, (double*)M->d, M->ld, N, N);
    stats_launch(ST_OTHER, 2);
    cudaFreeAsync(tmp, M->stream);
    cudaError_t e = cudaStreamSynchronize(M->stream);
    if (st == GBEM_OK && e != cudaSuccess) st = cuda_status(e, "F64 LU");
  } else {
    st = lu_factor_device(M->d, M->N, M->ld, M->dtype, M->d_ipiv, &h_info, M->stream, &M->ws, &M->ws_bytes);
  }
  if (st != GBEM_OK) return st;
  std::vector<int> piv(M->N), perm;
  CHECK_CUDA(cudaMemcpy(piv.data(), M->d_ipiv, sizeof(int) * M->N, cudaMemcpyDeviceToHost), "ipiv");
  perm_from_ipiv(piv, perm);
  CHECK_CUDA(cudaMemcpy(M->d_perm, perm.data(), sizeof(int) * M->N, cudaMemcpyHostToDevice), "perm");
  M->ipiv.resize(M->N);
  for (int i = 0; i < M->N; i++) M->ipiv[i] = piv[i] + 1;
  if (ipiv) memcpy(ipiv, M->ipiv.data(), sizeof(int) * M->N);
  if (info) *info = h_info;
  M->factored = true;
  if (h_info > 0) { set_error("LU: U(%d,%d) is exactly zero", h_info, h_info); return GBEM_ESINGULAR; }
  return GBEM_OK;
}

gbem_status gbem_lu_solve(gbem_matrix* M, char trans, int nrhs, void* B, int ldb) {
  if (!M || !B || nrhs <= 0 || ldb < M->N) { set_error("gbem_lu_solve: bad arguments"); return GBEM_EINVAL; }
  if (!M->factored) { set_error("gbem_lu_solve: matrix is not factored"); return GBEM_EINVAL; }
  CHECK_CUDA(cudaSetDevice(M->g->device), "cudaSetDevice");
  if (M->dtype == GBEM_F64) {
    // real factors: solved as complex128 with zero imaginary parts
    const int N = M->N;
    void *tA = nullptr, *dBr = nullptr, *dB = nullptr, *dY = nullptr;
    cudaStream_t s = M->stream;
    CHECK_CUDA(cudaMallocAsync(&tA, (size_t)N * N * 16, s), "solve alloc");
    CHECK_CUDA(cudaMallocAsync(&dBr, (size_t)N * nrhs * 8, s), "solve alloc");
    CHECK_CUDA(cudaMallocAsync(&dB, (size_t)N * nrhs * 16, s), "solve alloc");
    CHECK_CUDA(cudaMallocAsync(&dY, (size_t)N * 8 * 16, s), "solve alloc");
    CHECK_CUDA(cudaMemcpy2DAsync(dBr, (size_t)N * 8, B, (size_t)ldb * 8, (size_t)N * 8, nrhs, cudaMemcpyHostToDevice, s),
               "solve upload");
    make_complex<<<(unsigned)(((long long)N * N + 255) / 256), 256, 0, s>>>((const double*)M->d, M->ld, (double2*)tA, N,
                                                                            N, N);
    make_complex<<<(unsigned)(((long long)N * nrhs + 255) / 256), 256, 0, s>>>((const double*)dBr, N, (double2*)dB, N,
                                                                               N, nrhs);
    stats_launch(ST_OTHER, 3);
    gbem_status st = lu_solve_device(tA, N, N, GBEM_C128, M->d_perm, trans, nrhs, dB, N, dY, s);
    if (st == GBEM_OK) {
      take_real<<<(unsigned)(((long long)N * nrhs + 255) / 256), 256, 0, s>>>((const double2*)dB, N, (double*)dBr, N, N,
                                                                              nrhs);
      cudaError_t e = cudaMemcpy2DAsync(B, (size_t)ldb * 8, dBr, (size_t)N * 8, (size_t)N * 8, nrhs,
                                        cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) st = cuda_status(e, "solve download");
    }
    cudaFreeAsync(tA, s); cudaFreeAsync(dBr, s); cudaFreeAsync(dB, s); cudaFreeAsync(dY, s);
    cudaStreamSynchronize(s);
    return st;
  }
  size_t es = esize(M->dtype);
  void *dB = nullptr, *dY = nullptr;
  CHECK_CUDA(cudaMallocAsync(&dB, (size_t)M->N * nrhs * es, M->stream), "solve alloc");
  CHECK_CUDA(cudaMallocAsync(&dY, (size_t)M->N * 8 * es, M->stream), "solve alloc");
  CHECK_CUDA(cudaMemcpy2DAsync(dB, (size_t)M->N * es, B, (size_t)ldb * es, (size_t)M->N * es, nrhs,
                               cudaMemcpyHostToDevice, M->stream), "solve upload");
  gbem_status st = lu_solve_device(M->d, M->N, M->ld, M->dtype, M->d_perm, trans, nrhs, dB, M->N, dY, M->stream);
  if (st == GBEM_OK) {
    cudaError_t e = cudaMemcpy2DAsync(B, (size_t)ldb * es, dB, (size_t)M->N * es, (size_t)M->N * es, nrhs,
                                      cudaMemcpyDeviceToHost, M->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->stream);
    if (e != cudaSuccess) st = cuda_status(e, "solve download");
  }
  cudaFreeAsync(dB, M->stream);
  cudaFreeAsync(dY, M->stream);
  cudaStreamSynchronize(M->stream);
  return st;
}

// Tr over the first ncols diagonal entries of M^-1 B (GetTraceMInvdM,
// applications/scuff-cas3D/CasimirIntegrand.cc:100-146): B holds the
// derivative blocks of the BEM matrix in its first ncols columns.
static gbem_status trace_impl(gbem_matrix* M, const void* B, int ldb, int ncols, bool host, double* trace) {
  if (!M || !B || !trace || ncols <= 0 || ncols > M->N || ldb < M->N) {
    set_error("gbem_lu_trace: bad arguments");
    return GBEM_EINVAL;
  }
  if (!M->factored) { set_error("gbem_lu_trace: matrix is not factored"); return GBEM_EINVAL; }
  CHECK_CUDA(cudaSetDevice(M->g->device), "cudaSetDevice");
  const int N = M->N;
  cudaStream_t s = M->stream;
  const bool real = M->dtype == GBEM_F64;
  const int dt = real ? GBEM_C128 : M->dtype;           // element type of the solve
  const size_t es = dt == GBEM_C64 ? 8 : 16, ein = real ? 8 : es;
  void *A = M->d, *tA = nullptr, *X = nullptr, *tB = nullptr;
  double* d_out = nullptr;
  int lda = M->ld;
  gbem_status st = GBEM_OK;
  cudaError_t e = cudaMallocAsync(&X, (size_t)N * ncols * es, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_out, 2 * sizeof(double), s);
  if (e == cudaSuccess && real) e = cudaMallocAsync(&tA, (size_t)N * N * 16, s);
  if (e == cudaSuccess && real && host) e = cudaMallocAsync(&tB, (size_t)N * ncols * 8, s);
  if (e == cudaSuccess) {
    const void* src = B;
    long long lds = ldb;
    if (host) {
      // the host B goes through a device buffer: the real one, or X itself
      void* dst = real ? tB : X;
      e = cudaMemcpy2DAsync(dst, (size_t)N * ein, B, (size_t)ldb * ein, (size_t)N * ein, ncols, cudaMemcpyHostToDevice, s);
      src = dst;
      lds = N;
    } else if (!real) {
      e = cudaMemcpy2DAsync(X, (size_t)N * es, B, (size_t)ldb * es, (size_t)N * es, ncols, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess && real) {
      // real factors and B: solved as complex128 with zero imaginary parts
      make_complex<<<(unsigned)(((long long)N * N + 255) / 256), 256, 0, s>>>((const double*)M->d, M->ld, (double2*)tA,
                                                                              N, N, N);
      make_complex<<<(unsigned)(((long long)N * ncols + 255) / 256), 256, 0, s>>>((const double*)src, lds, (double2*)X,
                                                                                  N, N, ncols);
      stats_launch(ST_OTHER, 2);
      A = tA;
      lda = N;
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_trace setup");
  if (st == GBEM_OK) st = lu_solve_many_device(A, N, lda, dt, M->d_perm, ncols, X, N, s);
  if (st == GBEM_OK) {
    if (dt == GBEM_C64) trace_diag<float><<<1, 1024, 0, s>>>((const cx<float>*)X, N, ncols, d_out);
    else trace_diag<double><<<1, 1024, 0, s>>>((const cx<double>*)X, N, ncols, d_out);
    stats_launch(ST_OTHER);
    e = cudaMemcpyAsync(trace, d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_trace");
  }
  cudaFreeAsync(X, s); cudaFreeAsync(d_out, s);
  if (tA) cudaFreeAsync(tA, s);
  if (tB) cudaFreeAsync(tB, s);
  cudaStreamSynchronize(s);
  return st;
}

gbem_status gbem_lu_trace(gbem_matrix* M, const gbem_matrix* B, int ncols, double* trace) {
  if (!M || !B || B->N != M->N || B->dtype != M->dtype) {
    set_error("gbem_lu_trace: B must be a matrix of the same size and type as M");
    return GBEM_EINVAL;
  }
  return trace_impl(M, B->d, B->ld, ncols, false, trace);
}

gbem_status gbem_lu_trace_host(gbem_matrix* M, const void* B, int ldb, int ncols, double* trace) {
  return trace_impl(M, B, ldb, ncols, true, trace);
}

// ---- symmetric matrices in packed storage (LHM_SYMMETRIC) ----------------
gbem_status gbem_assemble_block_packed_host(gbem_geometry* g, int ns, double omega_re, double omega_im,
                                            const double* eps, const double* mu, void* AP, int dtype) {
  if (!g || !AP || ns < 0 || ns >= (int)g->S.size() || (dtype != GBEM_C128 && dtype != GBEM_F64)) {
    set_error("gbem_assemble_block_packed_host: bad arguments (dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  gbem_status st = ensure_stream(g);
  if (st != GBEM_OK) return st;
  CHECK_CUDA(cudaSetDevice(g->device), "cudaSetDevice");
  cudaStream_t s = g->stream;
  const int n = surface_bfs(g, ns);
  const size_t es = esize(dtype), np = (size_t)n * (n + 1) / 2;
  void *full = nullptr, *pk = nullptr;
  cudaError_t e = cudaMallocAsync(&full, (size_t)n * n * es, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&pk, np * es, s);
  if (e != cudaSuccess) st = cuda_status(e, "packed assembly alloc");
  BlockSel sel{ns, ns, 0, 0};
  if (st == GBEM_OK) st = assemble_into(g, omega_re, omega_im, eps, mu, GBEM_PREC_FP64, full, n, dtype, &sel);
  if (st == GBEM_OK) st = sp_pack_device(full, n, n, dtype, pk, s);
  if (st == GBEM_OK) {
    e = cudaMemcpyAsync(AP, pk, np * es, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "packed assembly download");
  }
  if (full) cudaFreeAsync(full, s);
  if (pk) cudaFreeAsync(pk, s);
  cudaStreamSynchronize(s);
  return st;
}

gbem_status gbem_sp_factor_host(void* AP, int N, int dtype, int* ipiv, int* info) {
  if (!AP || N <= 0 || (dtype != GBEM_C128 && dtype != GBEM_F64)) {
    set_error("gbem_sp_factor_host: bad arguments (N > 0, dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  const size_t es = esize(dtype), np = (size_t)N * (N + 1) / 2;
  cudaStream_t s;
  CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  void* dAP = nullptr;
  int* dpiv = nullptr;
  gbem_status st = GBEM_OK;
  int h_info = 0;
  cudaError_t e = cudaMallocAsync(&dAP, np * es, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dpiv, sizeof(int) * N, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dAP, AP, np * es, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = cuda_status(e, "gbem_sp_factor_host upload");
  if (st == GBEM_OK) st = sp_factor_device(dAP, N, dtype, dpiv, &h_info, s);
  if (st == GBEM_OK) {
    e = cudaMemcpyAsync(AP, dAP, np * es, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && ipiv) e = cudaMemcpyAsync(ipiv, dpiv, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_sp_factor_host download");
    if (info) *info = h_info;
  }
  if (dAP) cudaFreeAsync(dAP, s);
  if (dpiv) cudaFreeAsync(dpiv, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (st == GBEM_OK && h_info > 0) { set_error("sptrf: D(%d,%d) is exactly zero", h_info, h_info); return GBEM_ESINGULAR; }
  return st;
}

gbem_status gbem_sp_solve_host(const void* AP, int N, int dtype, const int* ipiv, int nrhs, void* B, int ldb) {
  if (!AP || !ipiv || !B || N <= 0 || nrhs <= 0 || ldb < N || (dtype != GBEM_C128 && dtype != GBEM_F64)) {
    set_error("gbem_sp_solve_host: bad arguments (dtype C128 or F64)");
    return GBEM_EINVAL;
  }
  // the solve walks the pivot codes downwards (1 x 1 steps, or 2 x 2 steps
  // over k-1, k) and upwards (k, k+1): both walks must stay inside [0, N)
  for (int k = 0; k < N; k++)
    if (ipiv[k] == 0 || ipiv[k] > N || ipiv[k] < -N) {
      set_error("gbem_sp_solve_host: ipiv[%d] = %d is not a pivot code of gbem_sp_factor_host", k, ipiv[k]);
      return GBEM_EINVAL;
    }
  for (int k = N - 1; k >= 0;) {
    if (ipiv[k] > 0) { k -= 1; continue; }
    if (k < 1 || ipiv[k - 1] != ipiv[k]) {
      set_error("gbem_sp_solve_host: ipiv[%d] = %d opens a 2 x 2 block without its partner", k, ipiv[k]);
      return GBEM_EINVAL;
    }
    k -= 2;
  }
  for (int k = 0; k < N;) {
    if (ipiv[k] > 0) { k += 1; continue; }
    if (k + 1 >= N || ipiv[k + 1] != ipiv[k]) {
      set_error("gbem_sp_solve_host: ipiv[%d] = %d opens a 2 x 2 block without its partner", k, ipiv[k]);
      return GBEM_EINVAL;
    }
    k += 2;
  }
  const size_t es = esize(dtype), np = (size_t)N * (N + 1) / 2;
  cudaStream_t s;
  CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  void *dAP = nullptr, *dB = nullptr;
  int* dpiv = nullptr;
  gbem_status st = GBEM_OK;
  cudaError_t e = cudaMallocAsync(&dAP, np * es, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dpiv, sizeof(int) * N, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&dB, (size_t)N * nrhs * es, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dAP, AP, np * es, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dpiv, ipiv, sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dB, (size_t)N * es, B, (size_t)ldb * es, (size_t)N * es, nrhs, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = cuda_status(e, "gbem_sp_solve_host upload");
  if (st == GBEM_OK) st = sp_solve_device(dAP, N, dtype, dpiv, nrhs, dB, N, s);
  if (st == GBEM_OK) {
    e = cudaMemcpy2DAsync(B, (size_t)ldb * es, dB, (size_t)N * es, (size_t)N * es, nrhs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_sp_solve_host download");
  }
  if (dAP) cudaFreeAsync(dAP, s);
  if (dpiv) cudaFreeAsync(dpiv, s);
  if (dB) cudaFreeAsync(dB, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return st;
}

gbem_status gbem_lu_tuning(int device, char* buf, int cap) {
  if (!buf || cap <= 0) { set_error("gbem_lu_tuning: NULL or empty buffer"); return GBEM_EINVAL; }
  int prev = 0;
  CHECK_CUDA(cudaGetDevice(&prev), "cudaGetDevice");
  CHECK_CUDA(cudaSetDevice(device), "cudaSetDevice");
  const std::string j = lu_tuning_json();
  cudaSetDevice(prev);  // the calling thread's current device is left as it was
  if ((int)j.size() + 1 > cap) { set_error("gbem_lu_tuning: %d bytes needed", (int)j.size() + 1); return GBEM_EINVAL; }
  memcpy(buf, j.c_str(), j.size() + 1);
  return GBEM_OK;
}

gbem_status gbem_lu_log_abs_det(gbem_matrix* M, double* logdet) {
  if (!M || !logdet) { set_error("gbem_lu_log_abs_det: NULL argument"); return GBEM_EINVAL; }
  if (!M->factored) { set_error("gbem_lu_log_abs_det: matrix is not factored"); return GBEM_EINVAL; }
  CHECK_CUDA(cudaSetDevice(M->g->device), "cudaSetDevice");
  cudaStream_t s = M->stream;
  double* d_out = nullptr;
  CHECK_CUDA(cudaMallocAsync((void**)&d_out, sizeof(double), s), "gbem_lu_log_abs_det alloc");
  if (M->dtype == GBEM_C64) log_abs_diag<float><<<1, 1024, 0, s>>>((const float*)M->d, M->ld, M->N, 1, d_out);
  else log_abs_diag<double><<<1, 1024, 0, s>>>((const double*)M->d, M->ld, M->N, M->dtype == GBEM_C128, d_out);
  stats_launch(ST_OTHER);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(logdet, d_out, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d_out, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = e2;
  return e == cudaSuccess ? GBEM_OK : cuda_status(e, "gbem_lu_log_abs_det");
}

gbem_status gbem_lu_solve_noalloc(gbem_matrix* M, char trans, int nrhs, void* B, int ldb) {
  if (!M || !B || nrhs <= 0 || ldb < M->N) { set_error("gbem_lu_solve_noalloc: bad arguments"); return GBEM_EINVAL; }
  CHECK_CUDA(cudaSetDevice(M->g->device), "cudaSetDevice");
  if (M->dtype == GBEM_F64)  // rejected with its reason before the size check
    return lu_solve_static_scratch(M->d, M->N, M->ld, M->dtype, M->d_perm, trans, nrhs, B, ldb, M->stream);
  if (M->N > lu_solve_noalloc_max_n(M->dtype)) {
    set_error("gbem_lu_solve_noalloc: N = %d exceeds the static scratch (N <= %d for this dtype)", M->N,
              lu_solve_noalloc_max_n(M->dtype));
    return GBEM_EINVAL;
  }
  if (!M->factored) { set_error("gbem_lu_solve_noalloc: matrix is not factored"); return GBEM_EINVAL; }
  return lu_solve_static_scratch(M->d, M->N, M->ld, M->dtype, M->d_perm, trans, nrhs, B, ldb, M->stream);
}

gbem_status gbem_lu_factor_host(double* ZM, int N, int ld, int* ipiv, int* info) {
  if (!ZM || N <= 0 || ld < N) { set_error("gbem_lu_factor_host: bad arguments"); return GBEM_EINVAL; }
  cudaStream_t s;
  CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  void* dA = nullptr;
  int* dpiv = nullptr;
  void* ws = nullptr;
  size_t wsb = 0;
  gbem_status st = GBEM_OK;
  cudaError_t e = cudaMalloc(&dA, (size_t)N * N * 16);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dpiv, sizeof(int) * N);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dA, (size_t)N * 16, ZM, (size_t)ld * 16, (size_t)N * 16, N, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_factor_host");
  int h_info = 0;
  if (st == GBEM_OK) st = lu_factor_device(dA, N, N, GBEM_C128, dpiv, &h_info, s, &ws, &wsb);
  if (st == GBEM_OK) {
    std::vector<int> piv(N);
    e = cudaMemcpy2DAsync(ZM, (size_t)ld * 16, dA, (size_t)N * 16, (size_t)N * 16, N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(piv.data(), dpiv, sizeof(int) * N, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_factor_host");
    else if (ipiv)
      for (int i = 0; i < N; i++) ipiv[i] = piv[i] + 1;
    if (info) *info = h_info;
  }
  cudaFree(dA); cudaFree(dpiv); cudaFree(ws);
  cudaStreamDestroy(s);
  if (st == GBEM_OK && h_info > 0) { set_error("LU: U(%d,%d) is exactly zero", h_info, h_info); return GBEM_ESINGULAR; }
  return st;
}

gbem_status gbem_lu_solve_host(const double* ZM, int N, int ld, const int* ipiv, char trans, int nrhs, double* B,
                               int ldb) {
  if (!ZM || !ipiv || !B || N <= 0 || ld < N || ldb < N || nrhs <= 0) {
    set_error("gbem_lu_solve_host: bad arguments");
    return GBEM_EINVAL;
  }
  std::vector<int> piv(N), perm;
  for (int i = 0; i < N; i++) {
    piv[i] = ipiv[i] - 1;
    if (piv[i] < i || piv[i] >= N) { set_error("gbem_lu_solve_host: invalid pivot %d at %d", ipiv[i], i + 1); return GBEM_EINVAL; }
  }
  perm_from_ipiv(piv, perm);
  cudaStream_t s;
  CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
  void *dA = nullptr, *dB = nullptr, *dY = nullptr;
  int* dperm = nullptr;
  gbem_status st = GBEM_OK;
  cudaError_t e = cudaMalloc(&dA, (size_t)N * N * 16);
  if (e == cudaSuccess) e = cudaMalloc(&dB, (size_t)N * nrhs * 16);
  if (e == cudaSuccess) e = cudaMalloc(&dY, (size_t)N * 8 * 16);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dperm, sizeof(int) * N);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dA, (size_t)N * 16, ZM, (size_t)ld * 16, (size_t)N * 16, N, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dB, (size_t)N * 16, B, (size_t)ldb * 16, (size_t)N * 16, nrhs, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dperm, perm.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_solve_host");
  if (st == GBEM_OK) st = lu_solve_device(dA, N, N, GBEM_C128, dperm, trans, nrhs, dB, N, dY, s);
  if (st == GBEM_OK) {
    e = cudaMemcpy2DAsync(B, (size_t)ldb * 16, dB, (size_t)N * 16, (size_t)N * 16, nrhs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_lu_solve_host");
  }
  cudaFree(dA); cudaFree(dB); cudaFree(dY); cudaFree(dperm);
  cudaStreamDestroy(s);
  return st;
}

// c64 <-> c128 conversions for the refinement loop
__global__ void to_c64(const double2* a, float2* b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void add_c64(double2* x, const float2* d, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) { x[i].x += (double)d[i].x; x[i].y += (double)d[i].y; }
}
__global__ void colnorm2(const double2* a, int N, int nrhs, double* out) {
  int r = blockIdx.x;
  double s = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) { double2 z = a[(size_t)r * N + i]; s += z.x * z.x + z.y * z.y; }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[r] = red[0];
}

__global__ void c64_to_c128(const float2* a, double2* b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_double2((double)a[i].x, (double)a[i].y);
}
__global__ void add_c128(double2* x, const double2* d, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) { x[i].x += d[i].x; x[i].y += d[i].y; }
}

// GMRES-based refinement, for matrices whose conditioning defeats plain
// refinement with the complex64 factor (kappa(A) u_f >~ 1: low frequencies,
// fine meshes).  Each outer step solves the correction equation A d = r,
// r = b - A x from the FP64 residual, by restarted GMRES(m) on the
// left-preconditioned system (LU)^-1 A d = (LU)^-1 r (Carson & Higham's
// GMRES-IR): products with A as in the residual (double-float accumulation
// on a complex64 matrix, FP64 on a complex128 one), the preconditioner by the
// complex64 triangular solves, the Krylov basis and the small Hessenberg
// problems on the host in FP64.  All right-hand sides advance together.
static gbem_status gmres_refine(const void* dA, int adtype, gbem_matrix* F, int N, int nrhs, const double2* dB,
                                double2* dX, double2* dR, float2* dD, void* dY, void* part, const std::vector<double>& bn,
                                double tol, int max_outer, int* iters, double* rel_out, cudaStream_t s) {
  typedef std::complex<double> C;
  const int m = 40;
  const size_t nel = (size_t)N * nrhs;
  const unsigned nb = (unsigned)((nel + 255) / 256);
  double2 *dV = nullptr, *dW = nullptr, *dZ = nullptr;
  double* dn = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dV, nel * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dW, nel * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dZ, nel * 16, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&dn, sizeof(double) * nrhs, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dZ, 0, nel * 16, s);
  gbem_status st = cuda_status(e, "GMRES workspace");
  std::vector<C> V((size_t)(m + 1) * nel), w(nel), H((size_t)(m + 1) * m * nrhs), g((size_t)(m + 1) * nrhs);
  std::vector<C> cs((size_t)m * nrhs), sn((size_t)m * nrhs);
  std::vector<double> rn(nrhs);
  // z = (LU)^-1 v for the nrhs columns of the device array src (complex128)
  auto precond = [&](const double2* src, std::vector<C>& out) -> gbem_status {
    to_c64<<<nb, 256, 0, s>>>(src, dD, nel);
    stats_launch(ST_OTHER);
    gbem_status q = lu_solve_device(F->d, N, N, GBEM_C64, F->d_perm, 'N', nrhs, dD, N, dY, s);
    if (q != GBEM_OK) return q;
    c64_to_c128<<<nb, 256, 0, s>>>(dD, dW, nel);
    stats_launch(ST_OTHER);
    cudaError_t ee = cudaMemcpyAsync(out.data(), dW, nel * 16, cudaMemcpyDeviceToHost, s);
    if (ee == cudaSuccess) ee = cudaStreamSynchronize(s);
    return cuda_status(ee, "GMRES preconditioner");
  };
  auto residual_norms = [&](double* rel) -> gbem_status {
    gbem_status q = residual_device(dA, N, adtype, N, (const double*)dX, N, (const double*)dB, N, nrhs, (double*)dR, N,
                                    part, s);
    if (q != GBEM_OK) return q;
    colnorm2<<<nrhs, 256, 0, s>>>(dR, N, nrhs, dn);
    stats_launch(ST_OTHER);
    cudaError_t ee = cudaMemcpyAsync(rn.data(), dn, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s);
    if (ee == cudaSuccess) ee = cudaStreamSynchronize(s);
    if (ee != cudaSuccess) return cuda_status(ee, "GMRES residual");
    *rel = 0.0;
    for (int r = 0; r < nrhs; r++) *rel = std::fmax(*rel, std::sqrt(rn[r] / (bn[r] > 0 ? bn[r] : 1.0)));
    return GBEM_OK;
  };
  double rel = *rel_out;
  for (int outer = 0; st == GBEM_OK && outer < max_outer && rel > tol; outer++) {
    // preconditioned residual, the first Krylov vector of every column
    std::vector<C> z(nel);
    st = precond(dR, z);
    if (st != GBEM_OK) break;
    std::vector<double> beta(nrhs);
    for (int c = 0; c < nrhs; c++) {
      double nz = 0.0;
      for (int i = 0; i < N; i++) nz += std::norm(z[(size_t)c * N + i]);
      beta[c] = std::sqrt(nz);
      for (int i = 0; i < N; i++) V[(size_t)c * N + i] = beta[c] > 0 ? z[(size_t)c * N + i] / beta[c] : C(0.0);
      for (int j = 0; j <= m; j++) g[(size_t)c * (m + 1) + j] = 0.0;
      g[(size_t)c * (m + 1)] = beta[c];
    }
    int kmax = 0;
    for (int j = 0; j < m; j++) {
      // w = (LU)^-1 A v_j: A v_j = -(0 - A v_j) by the residual kernel
      e = cudaMemcpyAsync(dV, V.data() + (size_t)j * nel, nel * 16, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) { st = cuda_status(e, "GMRES upload"); break; }
      st = residual_device(dA, N, adtype, N, (const double*)dV, N, (const double*)dZ, N, nrhs, (double*)dW, N, part, s);
      if (st != GBEM_OK) break;
      std::vector<C>& wv = w;
      // dW = -A v_j; precondition it (dW is overwritten by the result)
      e = cudaMemcpyAsync(dV, dW, nel * 16, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) { st = cuda_status(e, "GMRES copy"); break; }
      st = precond(dV, wv);
      if (st != GBEM_OK) break;
      bool all_small = true;
      for (int c = 0; c < nrhs; c++) {
        C* wc = wv.data() + (size_t)c * N;
        for (int i = 0; i < N; i++) wc[i] = -wc[i];
        C* Hc = H.data() + (size_t)c * (m + 1) * m;  // column-major (m+1) x m
        // modified Gram-Schmidt against v_0 .. v_j
        for (int i = 0; i <= j; i++) {
          const C* vi = V.data() + (size_t)i * nel + (size_t)c * N;
          C h = 0.0;
          for (int q = 0; q < N; q++) h += std::conj(vi[q]) * wc[q];
          Hc[i + (size_t)j * (m + 1)] = h;
          for (int q = 0; q < N; q++) wc[q] -= h * vi[q];
        }
        double hn = 0.0;
        for (int q = 0; q < N; q++) hn += std::norm(wc[q]);
        hn = std::sqrt(hn);
        Hc[j + 1 + (size_t)j * (m + 1)] = hn;
        C* vn = V.data() + (size_t)(j + 1) * nel + (size_t)c * N;
        for (int q = 0; q < N; q++) vn[q] = hn > 0 ? wc[q] / hn : C(0.0);
        // Givens rotations on column j of H and on g
        C* csc = cs.data() + (size_t)c * m;
        C* snc = sn.data() + (size_t)c * m;
        C* gc = g.data() + (size_t)c * (m + 1);
        for (int i = 0; i < j; i++) {
          const C a = Hc[i + (size_t)j * (m + 1)], b = Hc[i + 1 + (size_t)j * (m + 1)];
          Hc[i + (size_t)j * (m + 1)] = std::conj(csc[i]) * a + std::conj(snc[i]) * b;
          Hc[i + 1 + (size_t)j * (m + 1)] = -snc[i] * a + csc[i] * b;
        }
        const C a = Hc[j + (size_t)j * (m + 1)], b = Hc[j + 1 + (size_t)j * (m + 1)];
        const double den = std::sqrt(std::norm(a) + std::norm(b));
        csc[j] = den > 0 ? a / den : C(1.0);
        snc[j] = den > 0 ? b / den : C(0.0);
        Hc[j + (size_t)j * (m + 1)] = den;
        Hc[j + 1 + (size_t)j * (m + 1)] = 0.0;
        gc[j + 1] = -snc[j] * gc[j];
        gc[j] = std::conj(csc[j]) * gc[j];
        if (std::abs(gc[j + 1]) > 1e-7 * beta[c]) all_small = false;
      }
      kmax = j + 1;
      if (all_small) break;
    }
    if (st != GBEM_OK) break;
    // d = V y with H y = g (upper triangular, kmax x kmax), per column
    std::vector<C> d(nel, C(0.0));
    for (int c = 0; c < nrhs; c++) {
      C* Hc = H.data() + (size_t)c * (m + 1) * m;
      C* gc = g.data() + (size_t)c * (m + 1);
      std::vector<C> y(kmax);
      for (int i = kmax - 1; i >= 0; i--) {
        C t = gc[i];
        for (int k = i + 1; k < kmax; k++) t -= Hc[i + (size_t)k * (m + 1)] * y[k];
        const C piv = Hc[i + (size_t)i * (m + 1)];
        y[i] = std::abs(piv) > 0 ? t / piv : C(0.0);
      }
      for (int i = 0; i < kmax; i++) {
        const C* vi = V.data() + (size_t)i * nel + (size_t)c * N;
        for (int q = 0; q < N; q++) d[(size_t)c * N + q] += y[i] * vi[q];
      }
    }
    e = cudaMemcpyAsync(dV, d.data(), nel * 16, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { st = cuda_status(e, "GMRES correction"); break; }
    add_c128<<<nb, 256, 0, s>>>(dX, dV, nel);
    stats_launch(ST_OTHER);
    st = residual_norms(&rel);
    ++*iters;
  }
  cudaFreeAsync(dV, s); cudaFreeAsync(dW, s); cudaFreeAsync(dZ, s); cudaFreeAsync(dn, s);
  cudaStreamSynchronize(s);
  *rel_out = rel;
  return st;
}

// fp64_matrix: the matrix is assembled in FP64 (complex128), factored as its
// complex64 rounding, and the refinement residuals are taken against the
// complex128 matrix itself, so the solution converges to the FP64 solve's;
// otherwise the mixed assembly (float-float far field, complex64) is both
// factored and refined against.
static gbem_status solve_mixed_impl(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                    const double* mu, int nrhs, const void* B, int ldb, bool b_host, void* X, int ldx,
                                    bool x_host, double tol, int max_iter, int* iters, double* resid,
                                    bool fp64_matrix = false) {
  if (!g || !B || !X || nrhs <= 0 || nrhs > 64 || ldb < g->N || ldx < g->N) {
    set_error("gbem_solve_mixed: bad arguments");
    return GBEM_EINVAL;
  }
  gbem_status st0 = ensure_stream(g);
  if (st0 != GBEM_OK) return st0;
  const int N = g->N;
  cudaStream_t s = g->stream;
  // matrices and workspaces are cached on the geometry between solves
  gbem_status st = GBEM_OK;
  if (!g->mixedM || g->mixed_nrhs < nrhs) {
    if (g->mixedM) { gbem_matrix_destroy((gbem_matrix*)g->mixedM); gbem_matrix_destroy((gbem_matrix*)g->mixedF); }
    cudaFree(g->mixed_ws);
    g->mixedM = g->mixedF = nullptr;
    g->mixed_ws = nullptr;
    gbem_matrix *M = nullptr, *F = nullptr;
    st = gbem_matrix_create(g, GBEM_C64, &M);
    if (st == GBEM_OK) st = gbem_matrix_create(g, GBEM_C64, &F);
    if (st != GBEM_OK) return st;
    g->mixedM = M; g->mixedF = F;
    size_t wsb = (size_t)N * nrhs * 16 * 4 + (size_t)N * nrhs * 8 + (size_t)N * 8 * 8 +
                 (size_t)RESID_MAX_SPLIT * 8 * N * 16 + 4096;
    cudaError_t e = cudaMalloc(&g->mixed_ws, wsb);
    if (e != cudaSuccess) return cuda_status(e, "gbem_solve_mixed alloc");
    g->mixed_nrhs = nrhs;
  }
  gbem_matrix* M = (gbem_matrix*)g->mixedM;
  gbem_matrix* F = (gbem_matrix*)g->mixedF;
  unsigned char* w = (unsigned char*)g->mixed_ws;
  void* dB = w; w += (size_t)N * nrhs * 16;
  void* dX = w; w += (size_t)N * nrhs * 16;
  void* dR = w; w += (size_t)N * nrhs * 16;
  double* dn = (double*)w; w += (size_t)N * nrhs * 16;
  void* dD = w; w += (size_t)N * nrhs * 8;
  void* dY = w; w += (size_t)N * 8 * 8;
  void* part = w;
  cudaError_t e = cudaSuccess;
  gbem_matrix* M128 = nullptr;
  if (fp64_matrix) {
    st = gbem_matrix_create(g, GBEM_C128, &M128);
    if (st == GBEM_OK) st = gbem_assemble(g, omega_re, omega_im, eps, mu, GBEM_PREC_FP64, M128);
    if (st == GBEM_OK) {
      const size_t nn = (size_t)N * N;
      to_c64<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>((const double2*)M128->d, (float2*)F->d, nn);
      stats_launch(ST_OTHER);
      e = cudaGetLastError();
    }
  } else {
    st = gbem_assemble(g, omega_re, omega_im, eps, mu, GBEM_PREC_MIXED, M);
    if (st == GBEM_OK) e = cudaMemcpyAsync(F->d, M->d, (size_t)N * N * 8, cudaMemcpyDeviceToDevice, s);
  }
  if (st == GBEM_OK) {
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(dB, (size_t)N * 16, B, (size_t)ldb * 16, (size_t)N * 16, nrhs,
                            b_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dX, 0, (size_t)N * nrhs * 16, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dR, dB, (size_t)N * nrhs * 16, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_solve_mixed setup");
  }
  int info = 0;
  if (st == GBEM_OK) st = gbem_lu_factor(F, nullptr, &info);
  std::vector<double> bn(nrhs), rn(nrhs);
  if (st == GBEM_OK) {
    colnorm2<<<nrhs, 256, 0, s>>>((const double2*)dB, N, nrhs, dn);
    stats_launch(ST_OTHER);
    e = cudaMemcpyAsync(bn.data(), dn, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "norm");
  }
  int it = 0;
  double rel = 1.0;
  size_t nel = (size_t)N * nrhs;
  const void* dA = fp64_matrix ? M128->d : M->d;
  const int adt = fp64_matrix ? GBEM_C128 : GBEM_C64;
  // refinement sweeps x <- x + (LU)^-1 r, r = b - A x in FP64, until rel <=
  // tol; false when the sweeps stop contracting: plain refinement contracts
  // by ~kappa(A) u_f per sweep, and when that is not well below one (or the
  // residual grows) it will not reach tol
  auto refine = [&](int max_sweeps) -> bool {
    double prev = 2.0;
    for (int sw = 0; st == GBEM_OK && sw < max_sweeps; sw++) {
      to_c64<<<(unsigned)((nel + 255) / 256), 256, 0, s>>>((const double2*)dR, (float2*)dD, nel);
      stats_launch(ST_OTHER);
      {
        StatTimer t(ST_SOLVE, s);
        st = lu_solve_device(F->d, N, N, GBEM_C64, F->d_perm, 'N', nrhs, dD, N, dY, s);
      }
      if (st != GBEM_OK) break;
      add_c64<<<(unsigned)((nel + 255) / 256), 256, 0, s>>>((double2*)dX, (const float2*)dD, nel);
      stats_launch(ST_OTHER);
      {
        StatTimer t(ST_RESID, s);
        st = residual_device(dA, N, adt, N, (const double*)dX, N, (const double*)dB, N, nrhs, (double*)dR, N, part, s);
      }
      if (st != GBEM_OK) break;
      colnorm2<<<nrhs, 256, 0, s>>>((const double2*)dR, N, nrhs, dn);
      stats_launch(ST_OTHER);
      e = cudaMemcpyAsync(rn.data(), dn, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) { st = cuda_status(e, "refinement"); break; }
      it++;
      rel = 0;
      for (int r = 0; r < nrhs; r++) rel = std::fmax(rel, std::sqrt(rn[r] / (bn[r] > 0 ? bn[r] : 1.0)));
      if (rel <= tol) return true;
      if (sw >= 1 && !(rel < 0.2 * prev)) return false;
      prev = rel;
    }
    return rel <= tol;
  };
  bool ok = refine(max_iter);
  if (st == GBEM_OK && !ok) {
    // the split-BF16 factor is too coarse for this matrix: factor it again
    // with exact FP32 trailing updates (backward error ~1e-7 instead of
    // ~1e-4) and restart the refinement from x = 0
    if (fp64_matrix) {
      const size_t nn = (size_t)N * N;
      to_c64<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>((const double2*)M128->d, (float2*)F->d, nn);
      stats_launch(ST_OTHER);
      e = cudaGetLastError();
    } else {
      e = cudaMemcpyAsync(F->d, M->d, (size_t)N * N * 8, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(dX, 0, nel * 16, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dR, dB, nel * 16, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) st = cuda_status(e, "refactor");
    if (st == GBEM_OK) {
      tc_gemm_thread_off(1);
      st = gbem_lu_factor(F, nullptr, &info);
      tc_gemm_thread_off(0);
    }
    if (st == GBEM_OK) ok = refine(max_iter);
    // then GMRES-based refinement preconditioned by that factor
    if (st == GBEM_OK && !ok)
      st = gmres_refine(dA, adt, F, N, nrhs, (const double2*)dB, (double2*)dX, (double2*)dR, (float2*)dD, dY, part, bn,
                        tol, max_iter, &it, &rel, s);
  }
  if (st == GBEM_OK) {
    e = cudaMemcpy2DAsync(X, (size_t)ldx * 16, dX, (size_t)N * 16, (size_t)N * 16, nrhs,
                          x_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "gbem_solve_mixed download");
  }
  if (M128) gbem_matrix_destroy(M128);
  if (iters) *iters = it;
  if (resid) *resid = rel;
  if (st == GBEM_OK && rel > tol) {
    set_error("refinement stopped at relative residual %.3e after %d sweeps (tol %.1e)", rel, it, tol);
    return GBEM_ENOCONV;
  }
  return st;
}

gbem_status gbem_solve_mixed(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                             int nrhs, const double* B, int ldb, double* X, int ldx, double tol, int max_iter, int* iters,
                             double* resid) {
  return solve_mixed_impl(g, omega_re, omega_im, eps, mu, nrhs, B, ldb, true, X, ldx, true, tol, max_iter, iters, resid);
}

gbem_status gbem_solve_refined(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                               int nrhs, const double* B, int ldb, double* X, int ldx, double tol, int max_iter,
                               int* iters, double* resid) {
  return solve_mixed_impl(g, omega_re, omega_im, eps, mu, nrhs, B, ldb, true, X, ldx, true, tol, max_iter, iters, resid,
                          true);
}

gbem_status gbem_solve_mixed_batch(int njobs, gbem_batch_job* jobs, int max_concurrent) {
  if (njobs < 0 || (njobs > 0 && !jobs) || max_concurrent < 1) {
    set_error("gbem_solve_mixed_batch: bad arguments");
    return GBEM_EINVAL;
  }
  for (int i = 0; i < njobs; i++)
    if (!jobs[i].g) { set_error("gbem_solve_mixed_batch: job %d has no geometry", i); return GBEM_EINVAL; }
  // largest N first; one lock per geometry (its stream and cached buffers)
  std::vector<int> order(njobs);
  for (int i = 0; i < njobs; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].g->N > jobs[b].g->N; });
  std::map<gbem_geometry*, std::mutex> locks;
  for (int i = 0; i < njobs; i++) locks[jobs[i].g];
  std::atomic<int> next(0);
  std::vector<std::string> errs(njobs);
  auto worker = [&]() {
    for (;;) {
      const int q = next.fetch_add(1);
      if (q >= njobs) return;
      gbem_batch_job& j = jobs[order[q]];
      std::lock_guard<std::mutex> l(locks[j.g]);
      j.iters = 0;
      j.resid = 0.0;
      j.status = gbem_solve_mixed(j.g, j.omega_re, j.omega_im, j.eps, j.mu, j.nrhs, j.B, j.ldb, j.X, j.ldx, j.tol,
                                  j.max_iter, &j.iters, &j.resid);
      if (j.status != GBEM_OK && j.status != GBEM_ENOCONV) errs[order[q]] = gbem_last_error();
    }
  };
  const int nt = std::min(max_concurrent, std::max(njobs, 1));
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  gbem_status worst = GBEM_OK;
  int bad = -1;
  for (int i = 0; i < njobs; i++)
    if (jobs[i].status != GBEM_OK && jobs[i].status != GBEM_ENOCONV) { worst = jobs[i].status; if (bad < 0) bad = i; }
  if (bad >= 0) set_error("gbem_solve_mixed_batch: job %d: %s", bad, errs[bad].c_str());
  return worst;
}

gbem_status gbem_solve_mixed_device(gbem_geometry* g, double omega_re, double omega_im, const double* eps,
                                    const double* mu, int nrhs, const void* dB, int ldb, void* dX, int ldx, double tol,
                                    int max_iter, int* iters, double* resid) {
  return solve_mixed_impl(g, omega_re, omega_im, eps, mu, nrhs, dB, ldb, false, dX, ldx, false, tol, max_iter, iters,
                          resid);
}

gbem_status gbem_stats(int enable, double* ms, long long* counts) {
  if (g_stats_on) {
    for (int d = 0; d < 1; d++) cudaDeviceSynchronize();
  }
  stats_collect();
  {
    std::lock_guard<std::mutex> l(g_stats_mu);
    for (int i = 0; i < ST_N; i++) {
      if (ms) ms[i] = g_ms[i];
      if (counts) counts[i] = g_counts[i];
      g_ms[i] = 0;
      g_counts[i] = 0;
    }
    g_stats_on = enable != 0;
  }
  return GBEM_OK;
}

gbem_status gbem_rhs_planewave(gbem_geometry* g, double omega_re, double omega_im, const double* eps, const double* mu,
                               const double* E0, const double* nhat, double* rhs) {
  if (!g || !eps || !mu || !E0 || !nhat || !rhs) { set_error("gbem_rhs_planewave: NULL argument"); return GBEM_EINVAL; }
  gbem_status st0 = ensure_stream(g);
  if (st0 != GBEM_OK) return st0;
  void* d = nullptr;
  CHECK_CUDA(cudaMalloc(&d, sizeof(double) * 2 * g->N), "rhs alloc");
  gbem_status st = rhs_planewave_device(g, omega_re, omega_im, eps, mu, E0, nhat, d, g->stream);
  if (st == GBEM_OK) {
    cudaError_t e = cudaMemcpyAsync(rhs, d, sizeof(double) * 2 * g->N, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) st = cuda_status(e, "rhs download");
  }
  cudaFree(d);
  return st;
}

}  // extern "C"
