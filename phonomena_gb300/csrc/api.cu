// C ABI of libphono_gpu.so (declared in include/phono.h).
#include <cmath>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "../../include/phono.h"
#include <cudaTypedefs.h>
#include "fdtd_common.cuh"

namespace phono {
cudaError_t configure_step_f64(int tj);
cudaError_t configure_step_f32k(int tj);
cudaError_t launch_step_f64(const StepArgs<double>& a, int tj, int n_face_blocks, cudaStream_t st);
cudaError_t launch_step_f32k(const StepArgs<float>& a, int tj, int n_face_blocks, cudaStream_t st);
cudaError_t configure_step_f64v(int tj);
cudaError_t launch_step_f64v(const StepArgs<double>& a, int tj, int n_face_blocks, cudaStream_t st);
cudaError_t launch_energy(const EnergyArgs& a, double2* partial, int nblocks, double* out, cudaStream_t st);
cudaError_t batch_step_any(int precision, const void* ba, int tj, int grid_tiles, int grid_faces, cudaStream_t st);
cudaError_t batch_advance_any(int precision, const void* ba, int n_active_cap, int n, cudaStream_t st);
cudaError_t batch_configure_any(int precision, int tj, int* blocks_per_sm);
cudaError_t launch_lattice_ids(uint8_t* mat, const Geo& g, int pitch, int ncx, int ncy, const double* radius,
                               const uint8_t* kind, int depth, uint8_t host, cudaStream_t st);
cudaError_t launch_inclusion_ids(uint8_t* mat, const Geo& g, const double* x, const double* y, const double4* incl,
                                 const int* kend, const uint8_t* id, int n, uint8_t host, cudaStream_t st);

__global__ void advance_step_kernel(int* p, int n) { *p += n; }
// a batched instance's step counter, stopping at its budget
__global__ void advance_clamped_kernel(int* p, int n, int end) { *p = min(*p + n, end); }
}  // namespace phono

using namespace phono;

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

namespace phono {
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace phono

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static const int kGraphSteps = 12;  // multiple of 2 and 3: buffer rotations line up
static const int kEnergyBlocks = 1024;

struct phono_handle {
  phono_desc d;  // scalar copy; pointers not kept
  int es = 8;
  Geo g{};
  size_t field_elems = 0;  // per array
  size_t mat_bytes = 0;
  std::vector<void*> allocs;
  int nbuf = 3;            // u buffers: 3 rotating (F64) or 2 ping-pong (F32K)
  char* ubase = nullptr;   // nbuf x 3 padded arrays, buffer-major
  char* vbase = nullptr;   // F32K: 2 x 3 velocity arrays
  char* cbase = nullptr;   // F32K: 2 x 3 Kahan arrays
  CUtensorMap tm_u{}, tm_mat{}, tm_pw0{}, tm_pw1{};
  void* sp[6] = {};       // R spacings (F64 raw, F32K reciprocals)
  double* rsp64[6] = {};  // reciprocal double spacings 1/fd, 1/sd (energy)
  double h_sp0[6] = {};   // first elements (raw)
  DivTable dtab{};        // FP64 leapfrog: reciprocal pairs of the mesh's divisors (tab null: none)
  std::vector<double> sp_host[6];  // raw spacings (ABC coefficients)
  uint8_t* mat = nullptr;
  void* tab = nullptr;       // 16 R per material
  double* tab13 = nullptr;   // raw table (energy)
  double* src = nullptr;
  int nsrc = 0;
  void* surf = nullptr;
  int nrec_cap = 0;
  int* step_base = nullptr;
  int* err = nullptr;
  double2* partial = nullptr;
  double* energy_out = nullptr;
  double abc[8] = {};
  int tj = 8, xseg = 64, ntj = 0, ntk = 0, nseg = 0, n_tile = 0, n_face = 0, separate_faces = 1;
  FaceTable faces{};
  std::vector<int> seg_start;  // first plane of each x segment, + nx-1
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int steps_done = 0;
  int nmat = 0;
  bool timed = false;
  phono_batch* batch = nullptr;  // the batch that steps this handle, if any
  int wait_polls = 0;            // tile-pass wait budget (0: default)
  int skip_plane = -1;           // test hook of phono_test_wait_timeout (-1: off)
};

static long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

static int dalloc(phono_handle* h, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(PHONO_ERR_NOMEM, std::string("cudaMalloc ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
  }
  h->allocs.push_back(*p);
  return PHONO_OK;
}

static void batch_detach(phono_batch* b, const phono_handle* h);

static void release(phono_handle* h) {
  if (!h) return;
  if (h->batch) batch_detach(h->batch, h);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->allocs) cudaFree(p);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// ABC coefficients in the reference order from the material at node (0,0,0)
// (base_solver.py:525-537): clx[-1] ctx[-1] cty[0] cly[0] cty[-1] cly[-1] ctz[-1] clz[-1]
static void abc_coeffs(const phono_handle* h, const double* row0, double out[8]) {
  double vl = std::sqrt(row0[0] / row0[12]);
  double vt = std::sqrt(row0[9] / row0[12]);
  double vld = vl * h->d.dt, vtd = vt * h->d.dt;
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  const std::vector<double>&fdx = h->sp_host[0], &fdy = h->sp_host[1], &fdz = h->sp_host[2];
  const std::vector<double>&sdx = h->sp_host[3], &sdy = h->sp_host[4], &sdz = h->sp_host[5];
  out[0] = (vld - sdx[nx - 3]) / (vld + sdx[nx - 3]);
  out[1] = (vtd - fdx[nx - 2]) / (vtd + fdx[nx - 2]);
  out[2] = (vtd - fdy[0]) / (vtd + fdy[0]);
  out[3] = (vld - sdy[0]) / (vld + sdy[0]);
  out[4] = (vtd - fdy[ny - 2]) / (vtd + fdy[ny - 2]);
  out[5] = (vld - sdy[ny - 3]) / (vld + sdy[ny - 3]);
  out[6] = (vtd - fdz[nz - 2]) / (vtd + fdz[nz - 2]);
  out[7] = (vld - sdz[nz - 3]) / (vld + sdz[nz - 3]);
}

static int check_materials(const phono_handle* h, const uint8_t* mat, const double* table, int nmat) {
  if (!mat || !table) return fail(PHONO_ERR_ARG, "material ids or table is NULL");
  if (nmat < 1 || nmat > 256) return fail(PHONO_ERR_ARG, "nmat must be in 1..256");
  for (int q = 0; q < nmat * PHONO_TABLE_COLS; q++)
    if (!std::isfinite(table[q])) return fail(PHONO_ERR_ARG, "material table holds a non-finite value");
  for (int q = 0; q < nmat; q++)
    if (!(table[q * PHONO_TABLE_COLS + 12] > 0.0)) return fail(PHONO_ERR_ARG, "density must be > 0");
  size_t n = (size_t)h->d.nx * h->d.ny * h->d.nz;
  for (size_t q = 0; q < n; q++)
    if (mat[q] >= nmat) return fail(PHONO_ERR_ARG, "material id out of range");
  return PHONO_OK;
}

// ids into the padded layout, 16-entry device rows, raw rows, ABC coefficients
static int upload_table(phono_handle* h, const double* table, int nmat, int id000);

static int upload_materials(phono_handle* h, const uint8_t* mat, const double* table, int nmat) {
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  cudaMemcpy3DParms p{};
  p.srcPtr = make_cudaPitchedPtr((void*)mat, nz, nz, ny);
  p.dstPtr = make_cudaPitchedPtr(h->mat + h->g.mo0, h->g.msy, h->g.msy, ny + 2);
  p.extent = make_cudaExtent(nz, ny, nx);
  p.kind = cudaMemcpyHostToDevice;
  CK(cudaMemcpy3DAsync(&p, h->stream));
  return upload_table(h, table, nmat, mat[0]);
}

// the 16-entry device rows of the material table; id000 = the material at
// node (0, 0, 0), whose wave speeds set the absorbing-face coefficients
static int upload_table(phono_handle* h, const double* table, int nmat, int id000) {
  const double dt = h->d.dt;
  const double dt2 = dt * dt;
  if (h->es == 8) {
    const bool leapfrog = h->d.precision == PHONO_F64;
    std::vector<double> t(16 * nmat, 0.0);
    for (int m = 0; m < nmat; m++) {
      const double* row = table + m * PHONO_TABLE_COLS;
      for (int q = 0; q < 12; q++) t[m * 16 + q] = row[q];
      // (dt**2 / P) of base_solver.py:443 for the leapfrog, dt / P for the velocity form
      t[m * 16 + 12] = leapfrog ? dt2 / row[12] : dt / row[12];
      t[m * 16 + 13] = row[12];
      t[m * 16 + 14] = dt;
    }
    CK(cudaMemcpyAsync(h->tab, t.data(), t.size() * 8, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  } else {
    std::vector<float> t(16 * nmat, 0.0f);
    for (int m = 0; m < nmat; m++) {
      const double* row = table + m * PHONO_TABLE_COLS;
      for (int q = 0; q < 12; q++) t[m * 16 + q] = (float)row[q];
      t[m * 16 + 12] = (float)(dt / row[12]);
      t[m * 16 + 13] = (float)row[12];
      t[m * 16 + 14] = (float)dt;
    }
    CK(cudaMemcpyAsync(h->tab, t.data(), t.size() * 4, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  CK(cudaMemcpyAsync(h->tab13, table, (size_t)nmat * PHONO_TABLE_COLS * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->nmat = nmat;
  abc_coeffs(h, table + (size_t)id000 * PHONO_TABLE_COLS, h->abc);
  return PHONO_OK;
}

template <class R>
static StepArgs<R> make_args(const phono_handle* h, int step_off) {
  StepArgs<R> a{};
  a.g = h->g;
  a.sp.fdx = (const R*)h->sp[0];
  a.sp.fdy = (const R*)h->sp[1];
  a.sp.fdz = (const R*)h->sp[2];
  a.sp.sdx = (const R*)h->sp[3];
  a.sp.sdy = (const R*)h->sp[4];
  a.sp.sdz = (const R*)h->sp[5];
  R s0[6];
  // the leapfrog divides by raw spacings; the velocity forms multiply by reciprocals
  const bool raw = h->d.precision == PHONO_F64;
  for (int q = 0; q < 6; q++) s0[q] = raw ? (R)h->h_sp0[q] : (R)(1.0 / h->h_sp0[q]);
  a.sp.fdx0 = s0[0];
  a.sp.fdy0 = s0[1];
  a.sp.fdz0 = s0[2];
  a.sp.sdx0 = s0[3];
  a.sp.sdy0 = s0[4];
  a.sp.sdz0 = s0[5];
  a.dtab = h->dtab;
  a.mat = h->mat;
  a.tab = (const R*)h->tab;
  a.src = h->src;
  a.tm_u = h->tm_u;
  a.tm_mat = h->tm_mat;
  a.tm_pw0 = h->tm_pw0;
  a.tm_pw1 = h->tm_pw1;
  a.nmat = h->nmat;
  a.ubase = (R*)h->ubase;
  a.vbase = (R*)h->vbase;
  a.cbase = (R*)h->cbase;
  for (int q = 0; q < 8; q++) a.abc[q] = (R)h->abc[q];
  a.dt = (R)h->d.dt;
  a.surf = (R*)h->surf;
  a.record_every = h->d.record_every;
  a.rec_base = 0;
  a.nrec_cap = h->nrec_cap;
  a.step_base = h->step_base;
  a.step_off = step_off;
  a.surface_mode = h->d.surface_mode;
  a.bc = h->d.bc;
  a.source_mode = h->d.source_mode;
  a.ntj = h->ntj;
  a.ntk = h->ntk;
  a.nseg = h->nseg;
  for (int q = 0; q <= SEG_TABLE && q < (int)h->seg_start.size(); q++) a.seg_start[q] = h->seg_start[q];
  a.xseg = h->xseg;
  a.n_tile_blocks = h->n_tile;
  a.faces = h->faces;
  a.err = h->err;
  a.step_end = 0x7fffffff;
  a.wait_polls = h->wait_polls;
  a.skip_plane = h->skip_plane;
  return a;
}

// one time step (parts: the handle's form; or 2 tile launch only, 3 face launch only)
static cudaError_t launch_one(phono_handle* h, int step_off, int parts = -1) {
  const int form = parts < 0 ? h->separate_faces : parts;
  if (h->d.precision == PHONO_F64) return launch_step_f64(make_args<double>(h, step_off), h->tj, form, h->stream);
  if (h->d.precision == PHONO_F64V) return launch_step_f64v(make_args<double>(h, step_off), h->tj, form, h->stream);
  return launch_step_f32k(make_args<float>(h, step_off), h->tj, form, h->stream);
}

// Padded device layout: planes -1..nx, rows -1..ny, a KOFF-element front pad
// in z and rows rounded up to 128 bytes; material ids with an MKOFF front pad
// and 16-byte rows.
static long long field_row(int nz, int es) {
  const long long koff = es == 8 ? Lay<double>::KOFF : Lay<float>::KOFF;
  return round_up(koff + nz + 1, 128 / es);
}
static long long mat_row(int nz) { return round_up(MKOFF + nz + 1, 16); }

// Bytes of device memory phono_create allocates for a handle (each cudaMalloc
// rounded up to 512 bytes).
static size_t handle_bytes(int nx, int ny, int nz, int precision, int max_steps, int record_every) {
  const int es = precision == PHONO_F32K ? 4 : 8;
  const int nbuf = precision == PHONO_F64 ? 3 : 2;
  auto r = [](size_t b) { return (b + 511) / 512 * 512; };
  const size_t field_elems = (size_t)(nx + 2) * (ny + 2) * field_row(nz, es);
  const size_t fb = field_elems * es * 3 * nbuf;
  size_t total = r(fb) * (precision == PHONO_F64 ? 1 : 3);
  const int lens[6] = {nx - 1, ny - 1, nz - 1, nx - 2, ny - 2, nz - 2};
  for (int a = 0; a < 6; a++) total += r((size_t)(lens[a] + 3) * es) + r((size_t)lens[a] * 8);
  total += r((size_t)(nx + 2) * (ny + 2) * mat_row(nz));
  total += r((size_t)256 * 16 * es) + r((size_t)256 * PHONO_TABLE_COLS * 8);
  const int cap = max_steps > 0 ? max_steps : 1;
  total += r((size_t)cap * 8);
  const int nrec = record_every > 0 ? max_steps / record_every : 0;
  if (nrec > 0) total += r((size_t)nrec * nx * ny * es);
  total += r(sizeof(int) * 2) + r(sizeof(double2) * kEnergyBlocks) + r(sizeof(double) * 2);
  if (precision == PHONO_F64) total += r(sizeof(double) * 4 * DIV_TABLE_SLOTS_MAX);
  return total;
}

static int check_desc(const phono_desc* d) {
  if (!d) return fail(PHONO_ERR_ARG, "desc is NULL");
  if (d->nx < 3 || d->ny < 3 || d->nz < 3) return fail(PHONO_ERR_ARG, "nx, ny, nz must be >= 3 mesh nodes");
  if ((long long)d->nx * d->ny * d->nz > (1LL << 34)) return fail(PHONO_ERR_ARG, "grid too large");
  if (!d->fdx || !d->fdy || !d->fdz || !d->sdx || !d->sdy || !d->sdz) return fail(PHONO_ERR_ARG, "spacing array is NULL");
  if (!d->mat || !d->table) return fail(PHONO_ERR_ARG, "material ids or table is NULL");
  if (d->nmat < 1 || d->nmat > 256) return fail(PHONO_ERR_ARG, "nmat must be in 1..256");
  if (d->precision != PHONO_F64 && d->precision != PHONO_F32K && d->precision != PHONO_F64V)
    return fail(PHONO_ERR_ARG, "unknown precision");
  if (d->surface_mode < 0 || d->surface_mode > 1) return fail(PHONO_ERR_ARG, "unknown surface_mode");
  if (d->bc < 0 || d->bc > 1) return fail(PHONO_ERR_ARG, "unknown bc");
  if (d->source_mode < 0 || d->source_mode > 1) return fail(PHONO_ERR_ARG, "unknown source_mode");
  if (d->max_steps < 0 || d->record_every < 0) return fail(PHONO_ERR_ARG, "max_steps and record_every must be >= 0");
  if (!(d->dt > 0.0) || !std::isfinite(d->dt)) return fail(PHONO_ERR_ARG, "dt must be finite and > 0");
  if (d->tile_j != 0 && d->tile_j != 4 && d->tile_j != 8 && d->tile_j != 16) return fail(PHONO_ERR_ARG, "tile_j must be 0, 4, 8 or 16");
  if (d->x_segment < -4096) return fail(PHONO_ERR_ARG, "x_segment out of range");
  for (int q = 0; q < d->nmat * PHONO_TABLE_COLS; q++)
    if (!std::isfinite(d->table[q])) return fail(PHONO_ERR_ARG, "material table holds a non-finite value");
  for (int q = 0; q < d->nmat; q++)
    if (!(d->table[q * PHONO_TABLE_COLS + 12] > 0.0)) return fail(PHONO_ERR_ARG, "density must be > 0");
  const double* arrs[6] = {d->fdx, d->fdy, d->fdz, d->sdx, d->sdy, d->sdz};
  int lens[6] = {d->nx - 1, d->ny - 1, d->nz - 1, d->nx - 2, d->ny - 2, d->nz - 2};
  for (int a = 0; a < 6; a++)
    for (int q = 0; q < lens[a]; q++)
      if (!(arrs[a][q] > 0.0) || !std::isfinite(arrs[a][q])) return fail(PHONO_ERR_ARG, "spacings must be finite and > 0");
  size_t n = (size_t)d->nx * d->ny * d->nz;
  for (size_t q = 0; q < n; q++)
    if (d->mat[q] >= d->nmat) return fail(PHONO_ERR_ARG, "material id out of range");
  return PHONO_OK;
}

// 3-D copy between a dense host array (ex, ey, ez) and the padded device layout
static cudaError_t copy3d(phono_handle* h, void* dev, void* host, int c, bool to_dev) {
  int ex = h->d.nx - (c == 0), ey = h->d.ny - (c == 1), ez = h->d.nz - (c == 2);
  cudaMemcpy3DParms p{};
  cudaPitchedPtr hp = make_cudaPitchedPtr(host, (size_t)ez * h->es, (size_t)ez * h->es, ey);
  cudaPitchedPtr dp = make_cudaPitchedPtr((char*)dev + h->g.o0 * h->es, (size_t)h->g.sy * h->es,
                                          (size_t)h->g.sy * h->es, h->d.ny + 2);
  p.extent = make_cudaExtent((size_t)ez * h->es, ey, ex);
  if (to_dev) {
    p.srcPtr = hp;
    p.dstPtr = dp;
    p.kind = cudaMemcpyHostToDevice;
  } else {
    p.srcPtr = dp;
    p.dstPtr = hp;
    p.kind = cudaMemcpyDeviceToHost;
  }
  cudaError_t e = cudaMemcpy3DAsync(&p, h->stream);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(h->stream);
}

// buffers holding the current state after steps_done steps
static void* arr(const phono_handle* h, char* base, int buf, int comp) {
  return base + (size_t)(buf * 3 + comp) * h->field_elems * h->es;
}

static void* field_ptr(phono_handle* h, int field) {
  int t = h->steps_done;
  int comp = field % 3;
  if (h->d.precision == PHONO_F64) {
    if (field <= PHONO_FIELD_UZ) return arr(h, h->ubase, (t + 1) % 3, comp);
    if (field <= PHONO_FIELD_UZ_OLD) return arr(h, h->ubase, t % 3, comp);
    return nullptr;
  }
  int b = t & 1;
  if (field <= PHONO_FIELD_UZ) return arr(h, h->ubase, b, comp);
  if (field <= PHONO_FIELD_UZ_OLD) return nullptr;
  if (field <= PHONO_FIELD_VZ) return arr(h, h->vbase, b, comp);
  if (field <= PHONO_FIELD_CZ) return arr(h, h->cbase, b, comp);
  return nullptr;
}

// Tile decomposition of a handle: tile_j rows x 32 z-points per block, the
// x axis cut into segments of x_segment planes, and the face-pass work list.
// x_segment > 0: segments of x_segment planes (the last one shorter).
// x_segment = -L: tapered segments -- L planes while more than 2L planes are
// left, then the rest in four nearly equal parts -- so that the blocks a
// launch dispatches last are short and the tail of the last wave is short.
static std::vector<int> segment_starts(int planes, int xseg) {
  std::vector<int> st{0};
  if (xseg > 0) {
    for (int p = xseg; p < planes; p += xseg) st.push_back(p);
  } else {
    const int len = -xseg;
    int p = 0;
    while (planes - p > 2 * len) st.push_back(p += len);
    const int rem = planes - p, parts = rem >= 4 ? 4 : (rem > 0 ? rem : 0);
    for (int q = 1; q < parts; q++) st.push_back(p + (int)((long long)rem * q / parts));
  }
  st.push_back(planes);
  return st;
}

// h->xseg of a handle whose segments were given as a list (phono_set_segments)
constexpr int kExplicitSegments = INT_MIN;

// tile height tj and x segments starting at starts[0..n) (+ nx-1 at the end)
static int apply_tiling(phono_handle* h, int tj, int xseg, const std::vector<int>& starts) {
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  const int ntj = (ny - 1 + tj - 1) / tj, ntk = (nz - 1 + TK - 1) / TK, nseg = (int)starts.size() - 1;
  if (xseg <= 0 && nseg > SEG_TABLE) return fail(PHONO_ERR_ARG, "tapered or listed x segments: more than 64 segments");
  long long ntile = (long long)ntj * ntk * nseg;
  // face points left to the face pass, per component: z=N only where it meets
  // an x / y face (2*ex + ey-2; the tile pass writes the rest), y=N and y=0
  // (ex*(ez-1)), x=N ((ey-2)*(ez-1))
  FaceTable faces{};
  long long acc = 0;
  for (int c = 0; c < 3; c++) {
    long long ex = nx - (c == 0), ey = ny - (c == 1), ez = nz - (c == 2);
    long long cnt[4] = {2 * ex + (ey - 2), ex * (ez - 1), ex * (ez - 1), (ey - 2) * (ez - 1)};
    for (int p = 0; p < 4; p++) {
      faces.off[c * 4 + p] = (int)acc;
      acc += cnt[p];
    }
  }
  faces.off[12] = (int)acc;
  const long long nface = (acc + TK * tj - 1) / (TK * tj);
  if (ntile + nface > 0x7fffffffLL || acc > 0x7fffffffLL) return fail(PHONO_ERR_ARG, "grid too large for one launch");
  h->tj = tj;
  h->xseg = xseg;
  h->seg_start = starts;
  h->ntj = ntj;
  h->ntk = ntk;
  h->nseg = nseg;
  h->faces = faces;
  h->n_tile = (int)ntile;
  h->n_face = (int)nface;
  // faces in a second launch that reads the tile pass's interior values; the
  // chain end of a face point can itself be a face point only when ny == 3
  h->separate_faces = ny >= 4 ? 1 : 0;
  return PHONO_OK;
}

static int set_tiling(phono_handle* h, int tj, int xseg) {
  return apply_tiling(h, tj, xseg, segment_starts(h->d.nx - 1, xseg));
}

// TMA descriptors: a 4-D (k, j, i, array) map over the u allocation with a
// (KW, TJ+2, 1, 3) box (one plane tile of the three components of a buffer)
// and a 3-D (k, j, i) map over the material ids with a (48, TJ+2, 1) box.
static int encode_tensor_maps(phono_handle* h) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn) return fail(PHONO_ERR_CUDA, "cuTensorMapEncodeTiled not available");
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const int es = h->es;
  const int kw = es == 8 ? Lay<double>::KW : Lay<float>::KW;
  cuuint64_t dims[4] = {(cuuint64_t)h->g.sy, (cuuint64_t)(h->d.ny + 2), (cuuint64_t)(h->d.nx + 2),
                        (cuuint64_t)(h->nbuf * 3)};
  cuuint64_t strides[3] = {(cuuint64_t)h->g.sy * es, (cuuint64_t)h->g.sx * es, (cuuint64_t)h->field_elems * es};
  cuuint32_t box[4] = {(cuuint32_t)kw, (cuuint32_t)(h->tj + 2), 1, 3};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(&h->tm_u, es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                      h->ubase, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PHONO_ERR_CUDA, "cuTensorMapEncodeTiled (fields) failed: " + std::to_string(r));
  cuuint64_t mdims[3] = {(cuuint64_t)h->g.msy, (cuuint64_t)(h->d.ny + 2), (cuuint64_t)(h->d.nx + 2)};
  cuuint64_t mstr[2] = {(cuuint64_t)h->g.msy, (cuuint64_t)h->g.msx};
  cuuint32_t mbox[3] = {(cuuint32_t)MKW, (cuuint32_t)(h->tj + 2), 1};
  r = encode(&h->tm_mat, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, h->mat, mdims, mstr, mbox, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(PHONO_ERR_CUDA, "cuTensorMapEncodeTiled (materials) failed: " + std::to_string(r));
  // pointwise state, own points only: a (32, TJ, 1, 3) box over u_old (F64)
  // or over v and the Kahan terms (velocity forms)
  cuuint32_t pbox[4] = {(cuuint32_t)TK, (cuuint32_t)h->tj, 1, 3};
  const bool f64 = h->d.precision == PHONO_F64;
  void* pw[2] = {f64 ? h->ubase : h->vbase, f64 ? h->ubase : h->cbase};
  CUtensorMap* maps[2] = {&h->tm_pw0, &h->tm_pw1};
  for (int q = 0; q < 2; q++) {
    r = encode(maps[q], es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pw[q], dims,
               strides, pbox, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PHONO_ERR_CUDA, "cuTensorMapEncodeTiled (pointwise) failed: " + std::to_string(r));
  }
  return PHONO_OK;
}

extern "C" {

int phono_abi_version(void) { return PHONO_ABI_VERSION; }

int phono_footprint(int nx, int ny, int nz, int precision, int max_steps, int record_every, size_t* bytes) {
  if (!bytes) return fail(PHONO_ERR_ARG, "bytes is NULL");
  if (nx < 3 || ny < 3 || nz < 3) return fail(PHONO_ERR_ARG, "nx, ny, nz must be >= 3 mesh nodes");
  if ((long long)nx * ny * nz > (1LL << 34)) return fail(PHONO_ERR_ARG, "grid too large");
  if (precision != PHONO_F64 && precision != PHONO_F32K && precision != PHONO_F64V)
    return fail(PHONO_ERR_ARG, "unknown precision");
  if (max_steps < 0 || record_every < 0) return fail(PHONO_ERR_ARG, "max_steps and record_every must be >= 0");
  *bytes = handle_bytes(nx, ny, nz, precision, max_steps, record_every);
  return PHONO_OK;
}

const char* phono_last_error(void) { return g_err.c_str(); }

int phono_create(const phono_desc* d, phono_handle** out) {
  if (!out) return fail(PHONO_ERR_ARG, "out is NULL");
  *out = nullptr;
  int rc = check_desc(d);
  if (rc) return rc;
  phono_handle* h = new phono_handle();
  h->d = *d;
  h->d.fdx = h->d.fdy = h->d.fdz = h->d.sdx = h->d.sdy = h->d.sdz = nullptr;
  h->d.mat = nullptr;
  h->d.table = nullptr;
  const bool f64 = d->precision == PHONO_F64;  // leapfrog state (u_old, u, u_new)
  h->es = d->precision == PHONO_F32K ? 4 : 8;
  const int nx = d->nx, ny = d->ny, nz = d->nz;
  // padded layout: planes -1..nx, rows -1..ny, 32-byte front pad in z
  const long long koff = h->es == 8 ? Lay<double>::KOFF : Lay<float>::KOFF;
  const long long pz = field_row(nz, h->es);
  h->nbuf = f64 ? 3 : 2;
  h->g.nx = nx;
  h->g.ny = ny;
  h->g.nz = nz;
  h->g.sy = pz;
  h->g.sx = (long long)(ny + 2) * pz;
  h->g.o0 = h->g.sx + h->g.sy + koff;
  h->field_elems = (size_t)(nx + 2) * h->g.sx;
  if (h->field_elems >= (1ull << 32)) {  // the tile pass addresses an array with 32-bit offsets
    delete h;
    return fail(PHONO_ERR_ARG, "grid too large: one padded array exceeds 2^32 elements");
  }
  h->g.fstride = (long long)h->field_elems;
  const long long mpz = mat_row(nz);
  h->g.msy = mpz;
  h->g.msx = (long long)(ny + 2) * mpz;
  h->g.mo0 = h->g.msx + h->g.msy + MKOFF;
  h->mat_bytes = (size_t)(nx + 2) * h->g.msx;

  // tiles
  // default tile: height 4 for FP32 (one row a thread), 8 for FP64; 24 planes
  // per segment (the tuned shapes of the 256x256x128 crystal on GB300)
  if (set_tiling(h, d->tile_j ? d->tile_j : (d->precision == PHONO_F32K ? 4 : 8), d->x_segment ? d->x_segment : 24)) {
    std::string m_ = g_err;
    delete h;
    g_err = m_;
    return PHONO_ERR_ARG;
  }

  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return fail(PHONO_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
#define TRY(x)            \
  do {                    \
    int r_ = (x);         \
    if (r_) {             \
      std::string m_ = g_err; \
      release(h);         \
      g_err = m_;         \
      return r_;          \
    }                     \
  } while (0)
#define TRYC(x)                                                                         \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) {                                                            \
      release(h);                                                                       \
      return fail(PHONO_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));     \
    }                                                                                   \
  } while (0)
  TRYC(f64 ? configure_step_f64(h->tj)
           : (d->precision == PHONO_F64V ? configure_step_f64v(h->tj) : configure_step_f32k(h->tj)));
  TRYC(cudaEventCreate(&h->ev0));
  TRYC(cudaEventCreate(&h->ev1));
  const size_t fb = h->field_elems * h->es * 3 * h->nbuf;
  TRY(dalloc(h, (void**)&h->ubase, fb));
  TRYC(cudaMemsetAsync(h->ubase, 0, fb, h->stream));
  if (!f64) {
    TRY(dalloc(h, (void**)&h->vbase, fb));
    TRY(dalloc(h, (void**)&h->cbase, fb));
    TRYC(cudaMemsetAsync(h->vbase, 0, fb, h->stream));
    TRYC(cudaMemsetAsync(h->cbase, 0, fb, h->stream));
  }

  // spacings
  const double* arrs[6] = {d->fdx, d->fdy, d->fdz, d->sdx, d->sdy, d->sdz};
  int lens[6] = {nx - 1, ny - 1, nz - 1, nx - 2, ny - 2, nz - 2};
  // FP64 leapfrog: divisor table (div_tab in div_table.cuh) over the distinct
  // spacing values and 1.0, the divisors the step uses
  // (allocated for every FP64 handle, so that phono_footprint is exact)
  if (f64) {
    std::vector<double> tbl;
    double* tab_dev = nullptr;
    TRY(dalloc(h, (void**)&tab_dev, sizeof(double) * 4 * DIV_TABLE_SLOTS_MAX));
    std::vector<double> divisors{1.0};
    for (int a = 0; a < 6; a++) divisors.insert(divisors.end(), arrs[a], arrs[a] + lens[a]);
    if (build_div_table(divisors, tbl, &h->dtab.mult, &h->dtab.shift)) {
      TRYC(cudaMemcpy(tab_dev, tbl.data(), tbl.size() * sizeof(double), cudaMemcpyHostToDevice));
      h->dtab.tab = tab_dev;
    }
  }
  // device copies carry one value 1 before and two after the array, so the
  // tile pass reads the x spacings of its planes -1..nx without range tests
  // (the padding only reaches values whose results are discarded)
  for (int a = 0; a < 6; a++) {
    h->h_sp0[a] = arrs[a][0];
    h->sp_host[a].assign(arrs[a], arrs[a] + lens[a]);
    void* spb = nullptr;
    TRY(dalloc(h, &spb, (size_t)(lens[a] + 3) * h->es));
    h->sp[a] = (char*)spb + h->es;
    TRY(dalloc(h, (void**)&h->rsp64[a], (size_t)lens[a] * 8));
    {
      std::vector<double> rec(lens[a]);
      for (int q = 0; q < lens[a]; q++) rec[q] = 1.0 / arrs[a][q];
      TRYC(cudaMemcpy(h->rsp64[a], rec.data(), (size_t)lens[a] * 8, cudaMemcpyHostToDevice));
    }
    if (h->es == 8) {  // F64: raw spacings; F64V: reciprocals in double
      std::vector<double> r(lens[a] + 3, 1.0);
      for (int q = 0; q < lens[a]; q++) r[q + 1] = f64 ? arrs[a][q] : 1.0 / arrs[a][q];
      TRYC(cudaMemcpy(spb, r.data(), r.size() * 8, cudaMemcpyHostToDevice));
    } else {
      std::vector<float> r(lens[a] + 3, 1.0f);
      for (int q = 0; q < lens[a]; q++) r[q + 1] = (float)(1.0 / arrs[a][q]);
      TRYC(cudaMemcpy(spb, r.data(), r.size() * 4, cudaMemcpyHostToDevice));
    }
  }
  // materials: padded id layout and the 16-entry device rows (capacity 256 ids)
  TRY(dalloc(h, (void**)&h->mat, h->mat_bytes));
  TRYC(cudaMemset(h->mat, 0, h->mat_bytes));
  TRY(dalloc(h, &h->tab, (size_t)256 * 16 * h->es));
  TRY(dalloc(h, (void**)&h->tab13, (size_t)256 * PHONO_TABLE_COLS * 8));
  TRY(upload_materials(h, d->mat, d->table, d->nmat));
  TRY(encode_tensor_maps(h));
  // source table, surface records, counters
  int cap = d->max_steps > 0 ? d->max_steps : 1;
  TRY(dalloc(h, (void**)&h->src, (size_t)cap * 8));
  TRYC(cudaMemset(h->src, 0, (size_t)cap * 8));
  h->nrec_cap = d->record_every > 0 ? d->max_steps / d->record_every : 0;
  if (h->nrec_cap > 0) {
    size_t sb = (size_t)h->nrec_cap * nx * ny * h->es;
    TRY(dalloc(h, &h->surf, sb));
    TRYC(cudaMemsetAsync(h->surf, 0, sb, h->stream));
  }
  TRY(dalloc(h, (void**)&h->step_base, sizeof(int) * 2));
  h->err = h->step_base + 1;
  TRYC(cudaMemsetAsync(h->step_base, 0, sizeof(int) * 2, h->stream));
  TRY(dalloc(h, (void**)&h->partial, sizeof(double2) * kEnergyBlocks));
  TRY(dalloc(h, (void**)&h->energy_out, sizeof(double) * 2));
  TRYC(cudaStreamSynchronize(h->stream));
#undef TRY
#undef TRYC
  *out = h;
  return PHONO_OK;
}

int phono_set_source(phono_handle* h, const double* samples, int n) {
  if (!h || (!samples && n > 0)) return fail(PHONO_ERR_ARG, "NULL argument");
  if (n < 0 || n > (h->d.max_steps > 0 ? h->d.max_steps : 1)) return fail(PHONO_ERR_ARG, "n exceeds max_steps");
  for (int q = 0; q < n; q++)
    if (!std::isfinite(samples[q])) return fail(PHONO_ERR_ARG, "source sample is not finite");
  CK(cudaMemcpyAsync(h->src, samples, (size_t)n * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->nsrc = n;
  return PHONO_OK;
}

static int build_graph(phono_handle* h) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < kGraphSteps && e == cudaSuccess; s++) e = launch_one(h, s);
  if (e == cudaSuccess) {
    advance_step_kernel<<<1, 1, 0, h->stream>>>(h->step_base, kGraphSteps);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(PHONO_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  }
  if (e2 != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e2));
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return PHONO_OK;
}

int phono_step(phono_handle* h, int nsteps) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch: step it with phono_batch_step");
  if (nsteps < 0) return fail(PHONO_ERR_ARG, "nsteps < 0");
  if (h->steps_done + nsteps > h->nsrc)
    return fail(PHONO_ERR_STATE, "not enough source samples: call phono_set_source with max_steps samples");
  if (nsteps == 0) return PHONO_OK;
  if (!h->graph && nsteps >= kGraphSteps) {
    int rc = build_graph(h);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev0, h->stream));
  int full = nsteps / kGraphSteps, rem = nsteps % kGraphSteps;
  for (int q = 0; q < full; q++) CK(cudaGraphLaunch(h->graph, h->stream));
  for (int s = 0; s < rem; s++) CK(launch_one(h, s));
  if (rem) {
    advance_step_kernel<<<1, 1, 0, h->stream>>>(h->step_base, rem);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(h->ev1, h->stream));
  h->timed = true;
  h->steps_done += nsteps;
  return PHONO_OK;
}

int phono_time_kernels(phono_handle* h, int nsteps, float* tile_ms, float* face_ms) {
  if (!h || !tile_ms || !face_ms) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (nsteps < 1) return fail(PHONO_ERR_ARG, "nsteps must be >= 1");
  if (h->steps_done + nsteps > h->nsrc)
    return fail(PHONO_ERR_STATE, "not enough source samples: call phono_set_source with max_steps samples");
  const bool sep = h->separate_faces != 0;
  std::vector<cudaEvent_t> ev(3 * (size_t)nsteps, nullptr);
  cudaError_t e = cudaSuccess;
  for (size_t q = 0; q < ev.size() && e == cudaSuccess; q++) e = cudaEventCreate(&ev[q]);
  for (int s = 0; s < nsteps && e == cudaSuccess; s++) {
    e = cudaEventRecord(ev[3 * s], h->stream);
    if (e == cudaSuccess) e = launch_one(h, s, sep ? 2 : 0);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3 * s + 1], h->stream);
    if (e == cudaSuccess && sep) e = launch_one(h, s, 3);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3 * s + 2], h->stream);
  }
  if (e == cudaSuccess) {
    advance_step_kernel<<<1, 1, 0, h->stream>>>(h->step_base, nsteps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  float t = 0.f, f = 0.f;
  for (int s = 0; s < nsteps && e == cudaSuccess; s++) {
    float a = 0.f, b = 0.f;
    e = cudaEventElapsedTime(&a, ev[3 * s], ev[3 * s + 1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b, ev[3 * s + 1], ev[3 * s + 2]);
    t += a;
    f += b;
  }
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("phono_time_kernels: ") + cudaGetErrorString(e));
  h->steps_done += nsteps;
  *tile_ms = t;
  *face_ms = f;
  return PHONO_OK;
}

int phono_steps_done(const phono_handle* h) { return h ? h->steps_done : fail(PHONO_ERR_ARG, "handle is NULL"); }

// the device error word of a handle: bit 2 a tile-pass wait ran out, bit 1 a
// non-finite surface value
static int device_error(int err) {
  if (err & 2) return fail(PHONO_ERR_TIMEOUT, "a tile-pass pipeline wait ran out; the state of that step is invalid");
  if (err & 1) return fail(PHONO_ERR_NUMERIC, "non-finite value in the recorded surface");
  return PHONO_OK;
}

int phono_sync(phono_handle* h) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  CK(cudaStreamSynchronize(h->stream));
  int err = 0;
  CK(cudaMemcpy(&err, h->err, sizeof(int), cudaMemcpyDeviceToHost));
  return device_error(err);
}

int phono_test_wait_timeout(phono_handle* h, int polls, int skip_plane) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (polls < 0 || skip_plane < -1 || skip_plane > h->d.nx) return fail(PHONO_ERR_ARG, "polls >= 0, skip_plane in -1..nx");
  CK(cudaStreamSynchronize(h->stream));
  h->wait_polls = polls;
  h->skip_plane = skip_plane;
  if (h->graph) {  // the hook is a kernel argument baked into the graph
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return PHONO_OK;
}

int phono_last_step_ms(phono_handle* h, float* ms) {
  if (!h || !ms) return fail(PHONO_ERR_ARG, "NULL argument");
  if (!h->timed) return fail(PHONO_ERR_STATE, "no step timed yet");
  CK(cudaEventSynchronize(h->ev1));
  CK(cudaEventElapsedTime(ms, h->ev0, h->ev1));
  return PHONO_OK;
}

int phono_read_surface(phono_handle* h, int first, int count, void* host_out) {
  if (!h || (!host_out && count > 0)) return fail(PHONO_ERR_ARG, "NULL argument");
  if (first < 0 || count < 0 || first + count > h->nrec_cap) return fail(PHONO_ERR_ARG, "record range out of bounds");
  if (count == 0) return PHONO_OK;
  size_t rec = (size_t)h->d.nx * h->d.ny * h->es;
  CK(cudaMemcpyAsync(host_out, (char*)h->surf + (size_t)first * rec, (size_t)count * rec, cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return PHONO_OK;
}

int phono_set_steps_done(phono_handle* h, int steps) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (steps < 0 || steps > h->nsrc) return fail(PHONO_ERR_ARG, "steps must be in 0..(source samples set)");
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpy(h->step_base, &steps, sizeof(int), cudaMemcpyHostToDevice));
  h->steps_done = steps;
  return PHONO_OK;
}

int phono_upload_surface(phono_handle* h, int first, int count, const void* host_in) {
  if (!h || (!host_in && count > 0)) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (first < 0 || count < 0 || first + count > h->nrec_cap) return fail(PHONO_ERR_ARG, "record range out of bounds");
  if (count == 0) return PHONO_OK;
  size_t rec = (size_t)h->d.nx * h->d.ny * h->es;
  CK(cudaMemcpyAsync((char*)h->surf + (size_t)first * rec, host_in, (size_t)count * rec, cudaMemcpyHostToDevice,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return PHONO_OK;
}

static int field_check(phono_handle* h, int field, const void* host, size_t bytes, void** dev) {
  if (!h || !host) return fail(PHONO_ERR_ARG, "NULL argument");
  if (field < 0 || field > PHONO_FIELD_CZ) return fail(PHONO_ERR_ARG, "unknown field");
  *dev = field_ptr(h, field);
  if (!*dev) return fail(PHONO_ERR_ARG, "field not held by this precision");
  int c = field % 3;
  size_t n = (size_t)(h->d.nx - (c == 0)) * (h->d.ny - (c == 1)) * (h->d.nz - (c == 2));
  if (bytes != n * h->es) return fail(PHONO_ERR_ARG, "byte count does not match the field shape");
  return PHONO_OK;
}

int phono_download(phono_handle* h, int field, void* host, size_t bytes) {
  void* dev;
  int rc = field_check(h, field, host, bytes, &dev);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  CK(copy3d(h, dev, host, field % 3, false));
  return PHONO_OK;
}

int phono_upload(phono_handle* h, int field, const void* host, size_t bytes) {
  if (h && h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  void* dev;
  int rc = field_check(h, field, host, bytes, &dev);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  CK(copy3d(h, dev, (void*)host, field % 3, true));
  return PHONO_OK;
}

int phono_elem_size(const phono_handle* h) { return h ? h->es : fail(PHONO_ERR_ARG, "handle is NULL"); }

int phono_energy(phono_handle* h, double out[2]) {
  if (!h || !out) return fail(PHONO_ERR_ARG, "NULL argument");
  EnergyArgs a{};
  a.g = h->g;
  a.ux = field_ptr(h, PHONO_FIELD_UX);
  a.uy = field_ptr(h, PHONO_FIELD_UY);
  a.uz = field_ptr(h, PHONO_FIELD_UZ);
  const bool f64 = h->d.precision == PHONO_F64;
  a.vx = field_ptr(h, f64 ? PHONO_FIELD_UX_OLD : PHONO_FIELD_VX);
  a.vy = field_ptr(h, f64 ? PHONO_FIELD_UY_OLD : PHONO_FIELD_VY);
  a.vz = field_ptr(h, f64 ? PHONO_FIELD_UZ_OLD : PHONO_FIELD_VZ);
  a.f32 = h->es == 4 ? 1 : 0;
  a.vgiven = f64 ? 0 : 1;
  a.inv_dt = 1.0 / h->d.dt;
  a.rfdx = h->rsp64[0];
  a.rfdy = h->rsp64[1];
  a.rfdz = h->rsp64[2];
  a.rsdx = h->rsp64[3];
  a.rsdy = h->rsp64[4];
  a.rsdz = h->rsp64[5];
  a.mat = h->mat;
  a.tab = h->tab13;
  a.nmat = h->nmat;
  CK(launch_energy(a, h->partial, kEnergyBlocks, h->energy_out, h->stream));
  CK(cudaMemcpyAsync(out, h->energy_out, sizeof(double) * 2, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return PHONO_OK;
}

int phono_reset(phono_handle* h) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  const size_t fb = h->field_elems * h->es * 3 * h->nbuf;
  CK(cudaMemsetAsync(h->ubase, 0, fb, h->stream));
  if (h->vbase) CK(cudaMemsetAsync(h->vbase, 0, fb, h->stream));
  if (h->cbase) CK(cudaMemsetAsync(h->cbase, 0, fb, h->stream));
  if (h->surf) CK(cudaMemsetAsync(h->surf, 0, (size_t)h->nrec_cap * h->d.nx * h->d.ny * h->es, h->stream));
  CK(cudaMemsetAsync(h->step_base, 0, sizeof(int) * 2, h->stream));
  h->steps_done = 0;
  return PHONO_OK;
}

int phono_set_materials(phono_handle* h, const uint8_t* mat, const double* table, int nmat) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  int rc = check_materials(h, mat, table, nmat);
  if (rc) return rc;
  rc = upload_materials(h, mat, table, nmat);
  if (rc) return rc;
  // the absorbing-face coefficients are kernel arguments baked into the graph
  if (h->graph) {
    CK(cudaStreamSynchronize(h->stream));
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return PHONO_OK;
}

int phono_set_lattice(phono_handle* h, const phono_lattice* lat, const double* table, int nmat) {
  if (!h || !lat || !table || !lat->radius || !lat->kind) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (nmat < 1 || nmat > 256) return fail(PHONO_ERR_ARG, "nmat must be in 1..256");
  if (lat->pitch < 1 || lat->ncx < 1 || lat->ncy < 1) return fail(PHONO_ERR_ARG, "pitch and cell counts must be >= 1");
  if (lat->host < 0 || lat->host >= nmat) return fail(PHONO_ERR_ARG, "host material id out of range");
  const int ncell = lat->ncx * lat->ncy;
  for (int q = 0; q < ncell; q++) {
    if (lat->kind[q] >= nmat) return fail(PHONO_ERR_ARG, "hole material id out of range");
    if (!(lat->radius[q] >= 0.0) || !std::isfinite(lat->radius[q])) return fail(PHONO_ERR_ARG, "radius must be finite and >= 0");
  }
  for (int q = 0; q < nmat * PHONO_TABLE_COLS; q++)
    if (!std::isfinite(table[q])) return fail(PHONO_ERR_ARG, "material table holds a non-finite value");
  for (int q = 0; q < nmat; q++)
    if (!(table[q * PHONO_TABLE_COLS + 12] > 0.0)) return fail(PHONO_ERR_ARG, "density must be > 0");
  CK(cudaStreamSynchronize(h->stream));
  double* d_r = nullptr;
  uint8_t* d_k = nullptr;
  CK(cudaMalloc(&d_r, sizeof(double) * ncell));
  cudaError_t e = cudaMalloc(&d_k, ncell);
  if (e == cudaSuccess) e = cudaMemcpy(d_r, lat->radius, sizeof(double) * ncell, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_k, lat->kind, ncell, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_lattice_ids(h->mat, h->g, lat->pitch, lat->ncx, lat->ncy, d_r, d_k, lat->depth,
                                               (uint8_t)lat->host, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d_r);
  cudaFree(d_k);
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("lattice ids: ") + cudaGetErrorString(e));
  // node (0, 0, 0): inside the hole of cell (0, 0) only if its radius exceeds
  // the distance to the cell centre (the same test as the kernel's)
  const double c0 = 0.5 * lat->pitch, r0 = lat->radius[0];
  const int id000 = (c0 * c0 + c0 * c0 < r0 * r0 && lat->depth >= 0) ? lat->kind[0] : lat->host;
  int rc = upload_table(h, table, nmat, id000);
  if (rc) return rc;
  if (h->graph) {  // the absorbing-face coefficients are kernel arguments baked into the graph
    CK(cudaStreamSynchronize(h->stream));
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return PHONO_OK;
}

// z extent of each inclusion as simulation/grid.py:171-174 computes it.  The
// first inclusion keeps the z nodes with z <= t.z (the float32 depth widened
// to double).  That line rebinds the loop's `z` to the kept index array, so
// every later inclusion keeps the positions p of the previous selection with
// p <= t.z.  With ascending node coordinates every selection is a prefix of
// the z nodes: kend[t] is its length.
static std::vector<int> inclusion_z_extents(const double* z, int nz, const float* tz, int n) {
  std::vector<int> kend(n);
  int prev = nz;
  for (int t = 0; t < n; t++) {
    const double depth = (double)tz[t];
    int cnt = 0;
    if (t == 0) {
      for (int k = 0; k < nz; k++) cnt += z[k] <= depth;
    } else {
      for (int p = 0; p < prev; p++) cnt += (double)p <= depth;
    }
    kend[t] = cnt;
    prev = cnt;
  }
  return kend;
}

int phono_set_inclusions(phono_handle* h, const phono_inclusions* inc, const double* table, int nmat) {
  if (!h || !inc || !table || !inc->x || !inc->y || !inc->z) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz, n = inc->n;
  if (n < 0) return fail(PHONO_ERR_ARG, "n must be >= 0");
  if (n > 0 && (!inc->tx || !inc->ty || !inc->tz || !inc->tr)) return fail(PHONO_ERR_ARG, "NULL inclusion array");
  if (nmat < 1 || nmat > 256) return fail(PHONO_ERR_ARG, "nmat must be in 1..256");
  if (inc->host < 0 || inc->host >= nmat) return fail(PHONO_ERR_ARG, "host material id out of range");
  if (!inc->id && (inc->inside < 0 || inc->inside >= nmat)) return fail(PHONO_ERR_ARG, "inside material id out of range");
  for (int q = 0; q < n; q++)
    if (inc->id && inc->id[q] >= nmat) return fail(PHONO_ERR_ARG, "inclusion material id out of range");
  const double* axes[3] = {inc->x, inc->y, inc->z};
  const int ns[3] = {nx, ny, nz};
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < ns[a]; q++) {
      if (!std::isfinite(axes[a][q])) return fail(PHONO_ERR_ARG, "node coordinates must be finite");
      if (q > 0 && !(axes[a][q] > axes[a][q - 1])) return fail(PHONO_ERR_ARG, "node coordinates must ascend");
    }
  for (int q = 0; q < nmat * PHONO_TABLE_COLS; q++)
    if (!std::isfinite(table[q])) return fail(PHONO_ERR_ARG, "material table holds a non-finite value");
  for (int q = 0; q < nmat; q++)
    if (!(table[q * PHONO_TABLE_COLS + 12] > 0.0)) return fail(PHONO_ERR_ARG, "density must be > 0");
  const std::vector<int> kend = inclusion_z_extents(inc->z, nz, inc->tz, n);
  std::vector<double4> incl(n);
  std::vector<uint8_t> ids(n);
  for (int q = 0; q < n; q++) {
    incl[q] = make_double4((double)inc->tx[q], (double)inc->ty[q], (double)inc->tr[q], 0.0);
    ids[q] = inc->id ? inc->id[q] : (uint8_t)inc->inside;
  }
  // the material at node (0, 0, 0), by the kernel's test (its wave speeds set
  // the absorbing-face coefficients)
  int id000 = inc->host;
  for (int q = n - 1; q >= 0; q--) {
    if (kend[q] < 1) continue;
    const double dx = inc->x[0] - incl[q].x, dy = inc->y[0] - incl[q].y;
    if (std::sqrt(dx * dx + dy * dy) < incl[q].z) {
      id000 = ids[q];
      break;
    }
  }
  CK(cudaStreamSynchronize(h->stream));
  // one scratch allocation: coordinates, inclusions, extents, ids
  const size_t bx = (size_t)nx * 8, by = (size_t)ny * 8, bi = (size_t)n * sizeof(double4), bk = (size_t)n * 4;
  const size_t total = bx + by + bi + bk + n + 64;
  char* d = nullptr;
  CK(cudaMalloc(&d, total));
  double* dx = (double*)d;
  double* dy = (double*)(d + bx);
  double4* di = (double4*)(d + round_up(bx + by, 32));
  int* dk = (int*)((char*)di + bi);
  uint8_t* did = (uint8_t*)(dk + n);
  cudaError_t e = cudaMemcpy(dx, inc->x, bx, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dy, inc->y, by, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(di, incl.data(), bi, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(dk, kend.data(), bk, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(did, ids.data(), n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_inclusion_ids(h->mat, h->g, dx, dy, di, dk, did, n, (uint8_t)inc->host, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("inclusion ids: ") + cudaGetErrorString(e));
  int rc = upload_table(h, table, nmat, id000);
  if (rc) return rc;
  if (h->graph) {  // the absorbing-face coefficients are kernel arguments baked into the graph
    CK(cudaStreamSynchronize(h->stream));
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return PHONO_OK;
}

int phono_download_materials(phono_handle* h, uint8_t* host, size_t bytes) {
  if (!h || !host) return fail(PHONO_ERR_ARG, "NULL argument");
  const int nx = h->d.nx, ny = h->d.ny, nz = h->d.nz;
  if (bytes != (size_t)nx * ny * nz) return fail(PHONO_ERR_ARG, "byte count does not match nx*ny*nz");
  CK(cudaStreamSynchronize(h->stream));
  cudaMemcpy3DParms p{};
  p.srcPtr = make_cudaPitchedPtr(h->mat + h->g.mo0, h->g.msy, h->g.msy, ny + 2);
  p.dstPtr = make_cudaPitchedPtr((void*)host, nz, nz, ny);
  p.extent = make_cudaExtent(nz, ny, nx);
  p.kind = cudaMemcpyDeviceToHost;
  CK(cudaMemcpy3DAsync(&p, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return PHONO_OK;
}

void* phono_stream(phono_handle* h) { return h ? (void*)h->stream : nullptr; }

// switch a handle to tile height tj and the given x segments, keeping the old
// shape if the new one cannot be set up
static int retile(phono_handle* h, int tj, int xseg, const std::vector<int>& starts) {
  if (tj == h->tj && starts == h->seg_start) {
    h->xseg = xseg;
    return PHONO_OK;
  }
  CK(cudaStreamSynchronize(h->stream));
  const int p = h->d.precision;
  CK(p == PHONO_F64 ? configure_step_f64(tj) : (p == PHONO_F64V ? configure_step_f64v(tj) : configure_step_f32k(tj)));
  const int old_tj = h->tj, old_xs = h->xseg;
  const std::vector<int> old_starts = h->seg_start;
  int rc = apply_tiling(h, tj, xseg, starts);
  if (!rc) rc = encode_tensor_maps(h);
  if (rc) {
    std::string m = g_err;
    apply_tiling(h, old_tj, old_xs, old_starts);
    encode_tensor_maps(h);
    g_err = m;
    return rc;
  }
  if (h->graph) {  // the captured launches hold the old grid and tensor maps
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return PHONO_OK;
}

int phono_set_tiling(phono_handle* h, int tile_j, int x_segment) {
  if (!h) return fail(PHONO_ERR_ARG, "handle is NULL");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (tile_j == 0) tile_j = h->tj;
  if (tile_j != 4 && tile_j != 8 && tile_j != 16) return fail(PHONO_ERR_ARG, "tile_j must be 0, 4, 8 or 16");
  if (x_segment < -4096) return fail(PHONO_ERR_ARG, "x_segment out of range");
  if (x_segment == 0)  // keep the current segments (a list included)
    return retile(h, tile_j, h->xseg, h->seg_start);
  return retile(h, tile_j, x_segment, segment_starts(h->d.nx - 1, x_segment));
}

int phono_set_segments(phono_handle* h, int tile_j, const int* lengths, int n) {
  if (!h || !lengths) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_STATE, "handle is in a batch");
  if (tile_j == 0) tile_j = h->tj;
  if (tile_j != 4 && tile_j != 8 && tile_j != 16) return fail(PHONO_ERR_ARG, "tile_j must be 0, 4, 8 or 16");
  if (n < 1 || n > PHONO_MAX_SEGMENTS) return fail(PHONO_ERR_ARG, "n must be 1..PHONO_MAX_SEGMENTS");
  std::vector<int> starts{0};
  long long sum = 0;
  for (int q = 0; q < n; q++) {
    if (lengths[q] < 1) return fail(PHONO_ERR_ARG, "segment lengths must be >= 1");
    sum += lengths[q];
    if (sum > h->d.nx - 1) break;
    starts.push_back((int)sum);
  }
  if (sum != h->d.nx - 1) return fail(PHONO_ERR_ARG, "segment lengths must add up to nx - 1 planes");
  return retile(h, tile_j, kExplicitSegments, starts);
}

void phono_destroy(phono_handle* h) { release(h); }

}  // extern "C"

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
struct phono_batch {
  int cap = 0, precision = 0, tj = 8;
  size_t inst_size = 0;  // sizeof(StepArgs<R>)
  std::vector<void*> allocs;
  char* d_inst = nullptr;
  int2* d_items = nullptr;
  int item_cap = 0;
  int* d_counts = nullptr;  // items, face blocks, face entries, active instances
  unsigned* d_ticket = nullptr;
  int* d_face_prefix = nullptr;
  int* d_face_inst = nullptr;
  int* d_active = nullptr;
  std::vector<phono_handle*> slot;
  std::vector<int> remaining;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false, dirty = true;
  int grid_tiles = 0, grid_faces = 0;
  int streams = 0;  // PHONO_BATCH_STREAMS: per-instance launches on this many worker streams
  std::vector<cudaStream_t> workers;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  std::vector<int> order;     // active slots, costliest first
  std::vector<int> step_end;  // per slot: the instance's budget end
  std::vector<cudaGraphExec_t> igraph;  // streams scheme: per slot, 12 steps with its budget baked in
  cudaStream_t capture = nullptr;       // streams scheme: capture stream (always idle)
};

static void drop_igraph(phono_batch* b, int s) {
  if (s < (int)b->igraph.size() && b->igraph[s]) {
    cudaGraphExecDestroy(b->igraph[s]);
    b->igraph[s] = nullptr;
  }
}

// a handle destroyed while in a batch leaves it (the batch's work list is
// rebuilt before its next step)
static void batch_detach(phono_batch* b, const phono_handle* h) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (int s = 0; s < b->cap; s++)
    if (b->slot[s] == h) {
      b->slot[s] = nullptr;
      b->remaining[s] = 0;
      b->dirty = true;
      drop_igraph(b, s);
    }
}

static void batch_release(phono_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (phono_handle* h : b->slot)
    if (h) h->batch = nullptr;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (cudaGraphExec_t g : b->igraph)
    if (g) cudaGraphExecDestroy(g);
  for (void* p : b->allocs) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  for (cudaStream_t w : b->workers) cudaStreamDestroy(w);
  if (b->capture) cudaStreamDestroy(b->capture);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

static int balloc(phono_batch* b, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(PHONO_ERR_NOMEM, std::string("cudaMalloc ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
  }
  b->allocs.push_back(*p);
  return PHONO_OK;
}

// BatchArgs over the batch's device tables (same layout for float and double)
static BatchArgs<float> batch_args(const phono_batch* b, int step_off) {
  BatchArgs<float> ba{};
  ba.inst = reinterpret_cast<const StepArgs<float>*>(b->d_inst);
  ba.items = b->d_items;
  ba.counts = b->d_counts;
  ba.ticket = b->d_ticket;
  ba.face_prefix = b->d_face_prefix;
  ba.face_inst = b->d_face_inst;
  ba.active = b->d_active;
  ba.step_off = step_off;
  return ba;
}
static_assert(sizeof(BatchArgs<float>) == sizeof(BatchArgs<double>), "batch argument layouts differ");
static_assert(PHONO_MAX_SEGMENTS == SEG_TABLE, "segment list limit and the kernel table differ");

// work items (costliest instances first), face-block prefix, active list
static int batch_rebuild(phono_batch* b) {
  std::vector<int> act;
  for (int s = 0; s < b->cap; s++)
    if (b->slot[s] && b->remaining[s] > 0) act.push_back(s);
  // persistent scheme: the largest instances' work items first (the tail of
  // each step launch); streams scheme: the most remaining work first (node
  // updates left), each instance's chunks queued before the next one's
  auto cost = [&](int x) {
    const phono_handle* h = b->slot[x];
    return b->streams ? (long long)h->d.nx * h->d.ny * h->d.nz * b->remaining[x] : (long long)h->n_tile;
  };
  std::sort(act.begin(), act.end(), [&](int x, int y) {
    const long long cx = cost(x), cy = cost(y);
    return cx != cy ? cx > cy : x < y;
  });
  std::vector<int2> items;
  std::vector<int> prefix, finst;
  int fb = 0;
  for (int s : act) {
    const phono_handle* h = b->slot[s];
    for (int t = 0; t < h->n_tile; t++) items.push_back(make_int2(s, t));
    prefix.push_back(fb);
    finst.push_back(s);
    fb += (h->faces.off[12] + 255) / 256;
  }
  prefix.push_back(fb);
  b->order = act;
  if ((int)items.size() > b->item_cap) {
    int cap = std::max<int>((int)items.size(), 2 * b->item_cap);
    void* p = nullptr;
    int rc = balloc(b, &p, (size_t)cap * sizeof(int2));
    if (rc) return rc;
    b->d_items = (int2*)p;
    b->item_cap = cap;
    if (b->graph) {  // the captured launches hold the old pointer
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
  }
  int counts[4] = {(int)items.size(), fb, (int)finst.size(), (int)act.size()};
  if (!items.empty())
    CK(cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemcpyAsync(b->d_face_prefix, prefix.data(), prefix.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  if (!finst.empty()) {
    CK(cudaMemcpyAsync(b->d_face_inst, finst.data(), finst.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_active, act.data(), act.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  CK(cudaMemcpyAsync(b->d_counts, counts, sizeof counts, cudaMemcpyHostToDevice, b->stream));
  CK(cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned), b->stream));
  CK(cudaStreamSynchronize(b->stream));  // host vectors go out of scope
  b->dirty = false;
  return PHONO_OK;
}

// one step of instance s on stream st, with the handle's own kernels and tiles
static cudaError_t chain_launch(phono_batch* b, int s, int step_off, cudaStream_t st) {
  phono_handle* h = b->slot[s];
  if (h->d.precision == PHONO_F32K) {
    StepArgs<float> a = make_args<float>(h, step_off);
    a.step_end = b->step_end[s];
    return launch_step_f32k(a, h->tj, h->separate_faces, st);
  }
  StepArgs<double> a = make_args<double>(h, step_off);
  a.step_end = b->step_end[s];
  return h->d.precision == PHONO_F64 ? launch_step_f64(a, h->tj, h->separate_faces, st)
                                     : launch_step_f64v(a, h->tj, h->separate_faces, st);
}

static cudaError_t batch_launch_steps(phono_batch* b, int first_off, int n) {
  for (int s = 0; s < n; s++) {
    BatchArgs<float> ba = batch_args(b, first_off + s);
    cudaError_t e = batch_step_any(b->precision, &ba, b->tj, b->grid_tiles, b->grid_faces, b->stream);
    if (e != cudaSuccess) return e;
  }
  BatchArgs<float> ba = batch_args(b, 0);
  return batch_advance_any(b->precision, &ba, b->cap, n, b->stream);
}

// Streams scheme: the 12-step graph of the instance in slot s (its own step
// kernels, as phono_step launches them, and a step-counter update clamped at
// its budget), captured on the batch's idle capture stream
static int capture_instance(phono_batch* b, int s) {
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < kGraphSteps && e == cudaSuccess; q++) e = chain_launch(b, s, q, b->capture);
  if (e == cudaSuccess) {
    advance_clamped_kernel<<<1, 1, 0, b->capture>>>(b->slot[s]->step_base, kGraphSteps, b->step_end[s]);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamEndCapture(b->capture, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(PHONO_ERR_CUDA, std::string("instance graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(&b->igraph[s], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return PHONO_OK;
}

// Streams scheme: n steps of every active instance.  Instance q (costliest
// first) runs on worker q mod W; the host issues chunk by chunk (a 12-step
// instance graph each, then the remainder step by step) across the instances
// so that the workers progress together, and joins the workers back into the
// batch stream only after the last chunk: an instance's next chunk starts as
// soon as its previous one is done, whatever the others are doing.
static cudaError_t streams_steps(phono_batch* b, int n) {
  const int na = (int)b->order.size(), nw = std::min(na, b->streams);
  cudaError_t e = cudaEventRecord(b->fork, b->stream);
  for (int w = 0; w < nw && e == cudaSuccess; w++) e = cudaStreamWaitEvent(b->workers[w], b->fork, 0);
  const int full = n / kGraphSteps, rem = n % kGraphSteps;
  for (int c = 0; c < full && e == cudaSuccess; c++)
    for (int q = 0; q < na && e == cudaSuccess; q++) {
      const int s = b->order[q];
      if (b->remaining[s] > c * kGraphSteps) e = cudaGraphLaunch(b->igraph[s], b->workers[q % nw]);
    }
  for (int t = 0; t < rem && e == cudaSuccess; t++)
    for (int q = 0; q < na && e == cudaSuccess; q++) {
      const int s = b->order[q];
      if (b->remaining[s] > full * kGraphSteps + t) e = chain_launch(b, s, t, b->workers[q % nw]);
    }
  for (int q = 0; rem && q < na && e == cudaSuccess; q++) {
    const int s = b->order[q];
    if (b->remaining[s] <= full * kGraphSteps) continue;
    advance_clamped_kernel<<<1, 1, 0, b->workers[q % nw]>>>(b->slot[s]->step_base, rem, b->step_end[s]);
    e = cudaGetLastError();
  }
  for (int w = 0; w < nw && e == cudaSuccess; w++) {
    e = cudaEventRecord(b->joins[w], b->workers[w]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->joins[w], 0);
  }
  return e;
}

// Persistent scheme: 12-step graphs of the batch-wide launches (captured
// once: the launches read the work list from device memory), then the
// remainder step by step
static int persistent_steps(phono_batch* b, int nsteps) {
  if (!b->graph && nsteps >= kGraphSteps) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = batch_launch_steps(b, 0, kGraphSteps);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return fail(PHONO_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(PHONO_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  CK(cudaEventRecord(b->ev0, b->stream));
  const int full = nsteps / kGraphSteps, rem = nsteps % kGraphSteps;
  for (int q = 0; q < full; q++) CK(cudaGraphLaunch(b->graph, b->stream));
  if (rem) CK(batch_launch_steps(b, 0, rem));
  CK(cudaEventRecord(b->ev1, b->stream));
  return PHONO_OK;
}

extern "C" {

int phono_batch_create(int capacity, int precision, int tile_j, phono_batch** out) {
  if (!out) return fail(PHONO_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (capacity < 1 || capacity > (1 << 20)) return fail(PHONO_ERR_ARG, "capacity must be in 1..2^20");
  if (precision != PHONO_F64 && precision != PHONO_F32K && precision != PHONO_F64V)
    return fail(PHONO_ERR_ARG, "unknown precision");
  if (tile_j == 0) tile_j = 8;
  if (tile_j != 4 && tile_j != 8 && tile_j != 16) return fail(PHONO_ERR_ARG, "tile_j must be 4, 8 or 16");
  phono_batch* b = new phono_batch();
  b->cap = capacity;
  b->precision = precision;
  b->tj = tile_j;
  b->inst_size = precision == PHONO_F32K ? sizeof(StepArgs<float>) : sizeof(StepArgs<double>);
  b->slot.assign(capacity, nullptr);
  b->remaining.assign(capacity, 0);
  b->step_end.assign(capacity, 0);
  b->igraph.assign(capacity, nullptr);
#define BTRY(x)              \
  do {                       \
    int r_ = (x);            \
    if (r_) {                \
      std::string m_ = g_err; \
      batch_release(b);      \
      g_err = m_;            \
      return r_;             \
    }                        \
  } while (0)
#define BTRYC(x)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (x);                                                             \
    if (e_ != cudaSuccess) {                                                          \
      batch_release(b);                                                               \
      return fail(PHONO_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));   \
    }                                                                                 \
  } while (0)
  BTRYC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BTRYC(cudaEventCreate(&b->ev0));
  BTRYC(cudaEventCreate(&b->ev1));
  BTRY(balloc(b, (void**)&b->d_inst, b->inst_size * capacity));
  BTRY(balloc(b, (void**)&b->d_counts, sizeof(int) * 4));
  BTRY(balloc(b, (void**)&b->d_ticket, sizeof(unsigned)));
  BTRY(balloc(b, (void**)&b->d_face_prefix, sizeof(int) * (capacity + 1)));
  BTRY(balloc(b, (void**)&b->d_face_inst, sizeof(int) * capacity));
  BTRY(balloc(b, (void**)&b->d_active, sizeof(int) * capacity));
  BTRYC(cudaMemset(b->d_counts, 0, sizeof(int) * 4));
  BTRYC(cudaMemset(b->d_ticket, 0, sizeof(unsigned)));
  int bps = 0, dev = 0, nsm = 0;
  BTRYC(batch_configure_any(precision, tile_j, &bps));
  BTRYC(cudaGetDevice(&dev));
  BTRYC(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  b->grid_tiles = std::max(1, bps) * nsm;
  b->grid_faces = 8 * nsm;
#undef BTRY
#undef BTRYC
  *out = b;
  return PHONO_OK;
}

int phono_batch_set_mode(phono_batch* b, int mode, int streams) {
  if (!b) return fail(PHONO_ERR_ARG, "batch is NULL");
  if (mode != PHONO_BATCH_PERSISTENT && mode != PHONO_BATCH_STREAMS) return fail(PHONO_ERR_ARG, "unknown batch mode");
  if (mode == PHONO_BATCH_STREAMS && (streams < 1 || streams > 256))
    return fail(PHONO_ERR_ARG, "streams must be in 1..256");
  for (phono_handle* h : b->slot)
    if (h) return fail(PHONO_ERR_STATE, "the launch scheme of a batch is set while it is empty");
  CK(cudaStreamSynchronize(b->stream));
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  const int want = mode == PHONO_BATCH_STREAMS ? streams : 0;
  if (!b->fork && want) CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  if (!b->capture && want) CK(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
  while ((int)b->workers.size() < want) {  // worker streams are kept for the batch's lifetime
    cudaStream_t w = nullptr;
    cudaEvent_t j = nullptr;
    CK(cudaStreamCreateWithFlags(&w, cudaStreamNonBlocking));
    cudaError_t e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      cudaStreamDestroy(w);
      return fail(PHONO_ERR_CUDA, std::string("cudaEventCreateWithFlags: ") + cudaGetErrorString(e));
    }
    b->workers.push_back(w);
    b->joins.push_back(j);
  }
  b->streams = want;
  b->dirty = true;
  return PHONO_OK;
}

int phono_batch_add(phono_batch* b, phono_handle* h, int nsteps) {
  if (!b || !h) return fail(PHONO_ERR_ARG, "NULL argument");
  if (h->batch) return fail(PHONO_ERR_ARG, h->batch == b ? "handle already in the batch" : "handle is in another batch");
  if (h->d.precision != b->precision) return fail(PHONO_ERR_ARG, "handle precision differs from the batch");
  if (!b->streams && h->tj != b->tj) return fail(PHONO_ERR_ARG, "handle tile_j differs from the batch");
  if (!h->separate_faces) return fail(PHONO_ERR_ARG, "batched instances need ny >= 4");
  if (h->nmat > BATCH_TAB_ROWS)
    return fail(PHONO_ERR_ARG, "batched instances hold at most " + std::to_string(BATCH_TAB_ROWS) + " materials");
  if (nsteps < 0 || h->steps_done + nsteps > h->nsrc)
    return fail(PHONO_ERR_STATE, "not enough source samples for the requested steps");
  int s = -1;
  for (int q = 0; q < b->cap; q++) {
    if (b->slot[q] == h) return fail(PHONO_ERR_ARG, "handle already in the batch");
    if (s < 0 && !b->slot[q]) s = q;
  }
  if (s < 0) return fail(PHONO_ERR_NOMEM, "batch is full");
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (b->precision == PHONO_F32K) {
    StepArgs<float> a = make_args<float>(h, 0);
    a.step_end = h->steps_done + nsteps;
    CK(cudaMemcpy(b->d_inst + (size_t)s * b->inst_size, &a, sizeof a, cudaMemcpyHostToDevice));
  } else {
    StepArgs<double> a = make_args<double>(h, 0);
    a.step_end = h->steps_done + nsteps;
    CK(cudaMemcpy(b->d_inst + (size_t)s * b->inst_size, &a, sizeof a, cudaMemcpyHostToDevice));
  }
  b->slot[s] = h;
  b->remaining[s] = nsteps;
  b->step_end[s] = h->steps_done + nsteps;
  b->dirty = true;
  h->batch = b;
  return s;
}

int phono_batch_remove(phono_batch* b, int s) {
  if (!b || s < 0 || s >= b->cap || !b->slot[s]) return fail(PHONO_ERR_ARG, "no instance in that slot");
  CK(cudaStreamSynchronize(b->stream));
  b->slot[s]->batch = nullptr;
  b->slot[s] = nullptr;
  b->remaining[s] = 0;
  b->dirty = true;
  drop_igraph(b, s);
  return PHONO_OK;
}

int phono_batch_remaining(const phono_batch* b, int s) {
  if (!b || s < 0 || s >= b->cap || !b->slot[s]) return fail(PHONO_ERR_ARG, "no instance in that slot");
  return b->remaining[s];
}

int phono_batch_step(phono_batch* b, int nsteps) {
  if (!b) return fail(PHONO_ERR_ARG, "batch is NULL");
  if (nsteps < 0) return fail(PHONO_ERR_ARG, "nsteps < 0");
  if (nsteps == 0) return PHONO_OK;
  if (b->dirty) {
    for (int s = 0; s < b->cap; s++)
      if (b->slot[s]) CK(cudaStreamSynchronize(b->slot[s]->stream));
    int rc = batch_rebuild(b);
    if (rc) return rc;
  }
  if (b->streams) {
    if (nsteps >= kGraphSteps)
      for (int s : b->order)
        if (!b->igraph[s]) {
          int rc = capture_instance(b, s);
          if (rc) return rc;
        }
    CK(cudaEventRecord(b->ev0, b->stream));
    CK(streams_steps(b, nsteps));
    CK(cudaEventRecord(b->ev1, b->stream));
  } else {
    int rc = persistent_steps(b, nsteps);
    if (rc) return rc;
  }
  b->timed = true;
  for (int s = 0; s < b->cap; s++) {
    if (!b->slot[s] || b->remaining[s] <= 0) continue;
    const int adv = std::min(nsteps, b->remaining[s]);
    b->remaining[s] -= adv;
    b->slot[s]->steps_done += adv;
    if (b->remaining[s] == 0) b->dirty = true;
  }
  return PHONO_OK;
}

int phono_batch_sync(phono_batch* b) {
  if (!b) return fail(PHONO_ERR_ARG, "batch is NULL");
  CK(cudaStreamSynchronize(b->stream));
  for (int s = 0; s < b->cap; s++) {
    if (!b->slot[s]) continue;
    int err = 0;
    CK(cudaMemcpy(&err, b->slot[s]->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & 2) return fail(PHONO_ERR_TIMEOUT, "instance " + std::to_string(s) + ": a tile-pass pipeline wait ran out");
    if (err) return fail(PHONO_ERR_NUMERIC, "instance " + std::to_string(s) + ": non-finite surface value");
  }
  return PHONO_OK;
}

int phono_batch_last_step_ms(phono_batch* b, float* ms) {
  if (!b || !ms) return fail(PHONO_ERR_ARG, "NULL argument");
  if (!b->timed) return fail(PHONO_ERR_STATE, "no step timed yet");
  CK(cudaEventSynchronize(b->ev1));
  CK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
  return PHONO_OK;
}

void phono_batch_destroy(phono_batch* b) { batch_release(b); }

}  // extern "C"
