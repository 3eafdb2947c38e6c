// C ABI of libmsx.so (declared in include/msx.h): argument checks, plans,
// schedule tables and the multislice launch sequence.
#include "msx.h"
#include "msx_internal.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace msx;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(MSX_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

#define MSX_CUDA(call, what)                   \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

int schedule_table(int n, const SchedOps** ops) {
  switch (n) {
    case 64: return schedules_64(ops);
    case 128: return schedules_128(ops);
    case 256: return schedules_256(ops);
    case 384: return schedules_384(ops);
    case 512: return schedules_512(ops);
    case 768: return schedules_768(ops);
    case 1024: return schedules_1024(ops);
    default: *ops = nullptr; return 0;
  }
}

// cudaFuncSetAttribute must run once per device for every kernel of a schedule.
constexpr int kMaxDevices = 64;
constexpr int kMaxSchedPerSize = 8;
bool g_configured[kMaxDevices][8][kMaxSchedPerSize];

int size_slot(int n) {
  switch (n) {
    case 64: return 0; case 128: return 1; case 256: return 2; case 384: return 3;
    case 512: return 4; case 768: return 5; case 1024: return 6; default: return 7;
  }
}

int ensure_configured(int device, int n, int idx, const SchedOps& op) {
  if (device < 0 || device >= kMaxDevices || idx >= kMaxSchedPerSize) return fail(MSX_ERR_INVALID, "device/schedule index out of range");
  bool& done = g_configured[device][size_slot(n)][idx];
  if (!done) {
    MSX_CUDA(op.configure(), "configuring pass kernels");
    done = true;
  }
  return MSX_OK;
}

bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

}  // namespace

void msx::set_last_error(const char* msg) { g_err = msg; }

struct msx_plan {
  int ny = 0, nx = 0, device = 0;
  int group = 0;
  int row_sched = 0, col_sched = 0;
  const SchedOps* row_ops = nullptr;
  const SchedOps* col_ops = nullptr;
  float2* psi = nullptr;
  size_t psi_waves = 0;
  float2* ptab = nullptr;
  float2* tw_row = nullptr;
  float2* tw_col = nullptr;
  cudaStream_t work = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  bool use_graph = true;
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned char> gkey;
  cudaGraphExec_t gexec_host = nullptr;  // msx_multislice_host, page-locked buffers
  std::vector<unsigned char> gkey_host;
  // persistent TMA-pipelined passes
  bool use_tma = true;
  int* err = nullptr;            // device error word of the bounded waits
  float2* pyx = nullptr;         // py[ny] then px[nx]
  int2* band = nullptr;          // mask band per column
  CUtensorMap map{};             // workspace as (psi_waves*ny) x nx 8-byte elements, box col_c x col_boxr
  bool map_ok = false;
  int row_ctas = 0, col_ctas = 0;
  float* partial = nullptr;      // detector partial sums
  size_t partial_words = 0;
  float2* inv_n = nullptr;       // constant (1/N, 0) table for CBEDs of real-space waves
  // host-buffer calls (msx_multislice_host): a copy stream and device copies of
  // the inputs and of the CBED stack, grown as needed
  cudaStream_t copy = nullptr;
  cudaEvent_t ev_copy = nullptr;
  float2* io_trans = nullptr;
  size_t io_trans_words = 0;
  float2* io_psik = nullptr;
  size_t io_psik_words = 0;
  float* io_pos = nullptr;
  size_t io_pos_words = 0;
  double* io_norm = nullptr;
  float* io_cbed = nullptr;
  size_t io_cbed_words = 0;
};

namespace {

int upload_twiddles(const SchedOps& op, float2** dst) {
  std::vector<float2> h(op.tw_words > 0 ? op.tw_words : 1);
  op.host_twiddles(h.data());
  if (*dst) cudaFree(*dst);
  *dst = nullptr;
  cudaError_t e = cudaMalloc(dst, sizeof(float2) * h.size());
  if (e != cudaSuccess) return fail(MSX_ERR_ALLOC, "twiddle table allocation failed: %s", cudaGetErrorString(e));
  MSX_CUDA(cudaMemcpy(*dst, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice), "twiddle upload");
  return MSX_OK;
}

// Grows the wave workspace to `waves`.  The new buffer is allocated before the
// old one is released, so on failure the plan keeps its previous workspace.
int ensure_workspace(msx_plan* p, size_t waves) {
  if (waves <= p->psi_waves) return MSX_OK;
  float2* fresh = nullptr;
  cudaError_t e = cudaMalloc(&fresh, sizeof(float2) * waves * (size_t)p->ny * p->nx);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free allocation error
    return fail(MSX_ERR_ALLOC, "workspace of %zu waves (%d x %d) failed: %s", waves, p->ny, p->nx,
                cudaGetErrorString(e));
  }
  if (p->psi) cudaFree(p->psi);
  p->psi = fresh;
  p->psi_waves = waves;
  p->map_ok = false;  // the tensor map describes the old buffer until prepare_tma runs
  return MSX_OK;
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(f);
  }
  return fn;
}

// Tensor map of the wave workspace for the column pass's tile loads, and the
// persistent grid sizes of the current schedules.
int prepare_tma(msx_plan* p) {
  p->map_ok = false;
  EncodeTiled enc = encode_tiled();
  if (!enc) return fail(MSX_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)p->nx, (cuuint64_t)p->psi_waves * p->ny};
  const cuuint64_t strides[1] = {(cuuint64_t)p->nx * sizeof(float2)};
  const cuuint32_t box[2] = {(cuuint32_t)p->col_ops->col_c, (cuuint32_t)p->col_ops->col_boxr};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(&p->map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, p->psi, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MSX_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  int sms = 0, rr = 0, cr = 0, dummy = 0;
  MSX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device), "SM count");
  MSX_CUDA(p->row_ops->occupancy(&rr, &dummy), "occupancy");
  MSX_CUDA(p->col_ops->occupancy(&dummy, &cr), "occupancy");
  if (rr < 1 || cr < 1) return fail(MSX_ERR_CUDA, "persistent passes do not fit on an SM");
  p->row_ctas = sms * rr;
  p->col_ctas = sms * cr;
  p->map_ok = true;
  return MSX_OK;
}

void drop_graph(msx_plan* p) {
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  p->gexec = nullptr;
  p->gkey.clear();
  if (p->gexec_host) cudaGraphExecDestroy(p->gexec_host);
  p->gexec_host = nullptr;
  p->gkey_host.clear();
}

int auto_group(int ny, int nx) {
  // A resident group of about 1 GiB of waves (complex64), 4 to 512 waves: the
  // persistent passes run faster per wave on large groups than on groups small
  // enough to stay in L2 (tiles flow without launch tails); the plan autotuner
  // picks the same on GB300 for every supported grid.
  const size_t wave = sizeof(float2) * (size_t)ny * nx;
  size_t g = ((size_t)1 << 30) / wave;
  if (g < 4) g = 4;
  if (g > 512) g = 512;
  return (int)g;
}

// Schedules a plan starts with: the plan autotuner's choice on GB300 (random
// inputs, bandwidth 1/3, the groups above) -- the paired row transform for
// rows of 512, 16-column tiles for columns of 768, the first schedule
// elsewhere.
int schedule_index(int n, const char* name) {
  const SchedOps* ops = nullptr;
  const int k = schedule_table(n, &ops);
  for (int i = 0; i < k; ++i)
    if (std::strcmp(ops[i].name, name) == 0) return i;
  return 0;
}
int default_row_schedule(int nx) { return nx == 512 ? schedule_index(512, "t32_r16x2x16_pair") : 0; }
int default_col_schedule(int ny) { return ny == 768 ? schedule_index(768, "t32_r8x8x12_c16") : 0; }

struct MsArgs {
  const float* trans; int num_slices; const float* psik; const double* norm; const float* pos; int num_probes;
  float kmax; double lambda, slice_t; float k_band; float* cbed; int crop_y, crop_x;
  int group, row_sched, col_sched;
  const float* det; int ndet; float* signals;  // detector mode (det != nullptr): signals (P, ndet) instead of cbed
};

// One slice's row pass and (mid) column pass over a group of gn waves.
// Band-limited column range.  A column whose |kx| reaches the mask radius has
// |k| >= k_band for every ky, so the column pass zeroes it whole; from the second
// slice on those columns are zero on entry, stay zero through the row pass (which
// then need not write them) and need no column pass.  [x_lo, x_hi) is the range
// of column tiles (width C) holding every column with |kx| < k_band, with a
// 1e-6 relative margin on k_band so that it contains every column the device's
// float32 mask test keeps.  The whole grid when no column is in the band.
void band_columns(int nx, float kmax, float k_band, int C, int* x_lo, int* x_hi) {
  const double km = (double)kmax, lim = (double)k_band * (1.0 + 1e-6);
  int lo = nx, hi = -1;
  for (int j = 0; j < nx; ++j) {
    const double kx = (double)j * km / (double)(nx - 1) - km / 2.0;
    if (std::fabs(kx) < lim) {
      lo = j < lo ? j : lo;
      hi = j;
    }
  }
  if (hi < 0 || C <= 0) {
    *x_lo = 0;
    *x_hi = nx;
    return;
  }
  *x_lo = (lo / C) * C;
  *x_hi = (hi / C + 1) * C < nx ? (hi / C + 1) * C : nx;
}

// x_lo, x_hi: the column range of the TMA passes (0, 0 = all columns); the
// plain passes always cover every column.
int slice_passes(msx_plan* p, const float2* trans_s, int gn, const ColArgs& c, bool with_col, cudaStream_t st,
                 int x_lo = 0, int x_hi = 0) {
  if (p->use_tma && p->map_ok) {
    TmaPassArgs ta{};
    ta.psi = p->psi; ta.trans = trans_s; ta.tw = p->tw_row; ta.pyx = p->pyx; ta.band = p->band; ta.err = p->err;
    ta.G = gn; ta.Ny = p->ny; ta.Nx = p->nx; ta.x_lo = x_lo; ta.x_hi = x_hi;
    MSX_CUDA(p->row_ops->row_tma(ta, p->row_ctas, st), "row pass");
    if (with_col) {
      ta.tw = p->tw_col;
      MSX_CUDA(p->col_ops->col_tma(p->map, ta, p->col_ctas, st), "column pass");
    }
  } else {
    MSX_CUDA(p->row_ops->row(p->psi, trans_s, p->tw_row, gn, p->ny, st), "row pass");
    if (with_col) MSX_CUDA(p->col_ops->col(COL_MID, c, st), "column pass");
  }
  return MSX_OK;
}

// Copy pipeline of msx_multislice_host: the first group waits for each chunk of
// uploaded slices only when it reaches it, and each group's CBED block goes
// back to the host on the copy stream while the next group computes.
struct HostPipe {
  cudaStream_t copy;
  int chunk;                              // slices per upload chunk
  const std::vector<cudaEvent_t>* chunk_ev;  // recorded on the copy stream after each chunk
  std::vector<cudaEvent_t>* group_ev;        // recorded on the work stream after each group
  float* cbed_host;
  size_t pattern_words;                   // crop_y * crop_x
};

// A plan can only run groups its workspace holds (an allocation that failed
// leaves the previous workspace, or none).
bool workspace_holds(const msx_plan* p, int waves) { return p->psi && waves >= 0 && (size_t)waves <= p->psi_waves; }

// Grows a plan-owned device buffer of `words` elements of T.
template <class T>
int grow(T** buf, size_t* have, size_t words, const char* what) {
  if (words <= *have && *buf) return MSX_OK;
  T* fresh = nullptr;
  const cudaError_t e = cudaMalloc(&fresh, sizeof(T) * (words ? words : 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(MSX_ERR_ALLOC, "%s: allocation of %zu bytes failed", what, sizeof(T) * words);
  }
  if (*buf) cudaFree(*buf);
  *buf = fresh;
  *have = words;
  return MSX_OK;
}

int enqueue_multislice(msx_plan* p, const MsArgs& a, cudaStream_t st, const HostPipe* hp = nullptr) {
  const int ny = p->ny, nx = p->nx;
  const int gmax = a.num_probes < a.group ? a.num_probes : a.group;
  if (!workspace_holds(p, gmax))
    return fail(MSX_ERR_ALLOC, "the plan's workspace does not hold %d waves (an earlier allocation failed)", gmax);
  MSX_CUDA(launch_ptab(ny, nx, a.kmax, a.lambda, a.slice_t, a.k_band, p->ptab, st), "propagator table");
  if (p->use_tma && p->map_ok)
    MSX_CUDA(launch_pfac(ny, nx, a.kmax, a.lambda, a.slice_t, a.k_band, p->pyx, p->band, st), "propagator factors");
  const size_t wave = (size_t)ny * nx;
  const int y0 = ny / 2 - a.crop_y / 2, x0 = nx / 2 - a.crop_x / 2;
  const float2* trans = reinterpret_cast<const float2*>(a.trans);
  int bx_lo = 0, bx_hi = 0;
  band_columns(nx, a.kmax, a.k_band, p->col_ops->col_c, &bx_lo, &bx_hi);
  // group done: hand its CBED block to the copy stream (host-buffer calls)
  auto hand_off = [&](int gi, int g0, int gn) -> int {
    if (!hp) return MSX_OK;
    cudaEvent_t ev = (*hp->group_ev)[gi];
    MSX_CUDA(cudaEventRecord(ev, st), "cudaEventRecord");
    MSX_CUDA(cudaStreamWaitEvent(hp->copy, ev, 0), "cudaStreamWaitEvent");
    MSX_CUDA(cudaMemcpyAsync(hp->cbed_host + (size_t)g0 * hp->pattern_words, a.cbed + (size_t)g0 * hp->pattern_words,
                             sizeof(float) * (size_t)gn * hp->pattern_words, cudaMemcpyDeviceToHost, hp->copy),
             "CBED download");
    return MSX_OK;
  };
  for (int g0 = 0, gi = 0; g0 < a.num_probes; g0 += a.group, ++gi) {
    const int gn = (a.num_probes - g0 < a.group) ? a.num_probes - g0 : a.group;
    ColArgs c{};
    c.psi = p->psi;
    c.ptab = p->ptab;
    c.psik = reinterpret_cast<const float2*>(a.psik);
    c.pos_yx = a.pos + 2 * (size_t)g0;
    c.tw = p->tw_col;
    c.norm = a.norm;
    c.cbed = a.cbed + (size_t)g0 * a.crop_y * a.crop_x;
    c.G = gn;
    c.Nx = nx;
    c.kmax = a.kmax;
    c.y0 = y0;
    c.crop_y = a.crop_y;
    if (a.num_slices == 0) {
      c.x_begin = x0;
      c.ncols = a.crop_x;
      MSX_CUDA(p->col_ops->col(COL_INIT_FINAL, c, st), "probe-only pass");
      const int rc = hand_off(gi, g0, gn);
      if (rc != MSX_OK) return rc;
      continue;
    }
    c.x_begin = 0;
    c.ncols = nx;
    MSX_CUDA(p->col_ops->col(COL_INIT, c, st), "probe formation pass");
    for (int s = 0; s < a.num_slices; ++s) {
      if (hp && gi == 0 && s % hp->chunk == 0)
        MSX_CUDA(cudaStreamWaitEvent(st, (*hp->chunk_ev)[s / hp->chunk], 0), "cudaStreamWaitEvent");
      // the first slice covers every column (the probe may reach beyond the band)
      const int rc = slice_passes(p, trans + (size_t)s * wave, gn, c, s + 1 < a.num_slices, st, s > 0 ? bx_lo : 0,
                                  s > 0 ? bx_hi : 0);
      if (rc != MSX_OK) return rc;
      if (s + 1 == a.num_slices) {
        ColArgs f = c;
        if (a.det) {
          f.det = a.det;
          f.ndet = a.ndet;
          f.partial = p->partial;
          MSX_CUDA(p->col_ops->col(COL_DETECT, f, st), "detector pass");
          MSX_CUDA(launch_detect_reduce(p->partial, gn, nx / p->col_ops->col_c, a.ndet,
                                        a.signals + (size_t)g0 * a.ndet, st), "detector reduction");
        } else {
          f.x_begin = x0;
          f.ncols = a.crop_x;
          MSX_CUDA(p->col_ops->col(COL_FINAL, f, st), "final column pass");
          const int rc2 = hand_off(gi, g0, gn);
          if (rc2 != MSX_OK) return rc2;
        }
      }
    }
  }
  return MSX_OK;
}

}  // namespace

extern "C" {

int msx_version(void) { return 1 * 10000 + 0 * 100 + 0; }

int msx_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_err.c_str(), len - 1);
    buf[len - 1] = '\0';
  }
  return (int)g_err.size();
}

int msx_supported_size(int n) {
  const SchedOps* ops;
  return schedule_table(n, &ops) > 0 ? 1 : 0;
}

int msx_num_schedules(int n) {
  const SchedOps* ops;
  return schedule_table(n, &ops);
}

int msx_schedule_name(int n, int index, char* buf, size_t len) {
  const SchedOps* ops;
  const int cnt = schedule_table(n, &ops);
  if (index < 0 || index >= cnt) return fail(MSX_ERR_INVALID, "no schedule %d for length %d", index, n);
  if (buf && len) {
    std::strncpy(buf, ops[index].name, len - 1);
    buf[len - 1] = '\0';
  }
  return MSX_OK;
}

int msx_schedule_col_tile(int n, int index, int* tile) {
  const SchedOps* ops;
  const int cnt = schedule_table(n, &ops);
  if (index < 0 || index >= cnt || !tile) return fail(MSX_ERR_INVALID, "no schedule %d for length %d", index, n);
  *tile = ops[index].col_c;
  return MSX_OK;
}

int msx_band_columns(int nx, float kmax, float k_band, int tile, int* x_lo, int* x_hi) {
  if (nx <= 1 || tile <= 0 || !x_lo || !x_hi || !(kmax > 0)) return fail(MSX_ERR_INVALID, "band_columns arguments");
  band_columns(nx, kmax, k_band, tile, x_lo, x_hi);
  return MSX_OK;
}

int msx_atom_windows(const double* coeff_dev, int nspecies, int n0, int n1, int oversample, double potential_range,
                     float* windows_out_dev, void* stream) {
  if (!coeff_dev || !windows_out_dev) return fail(MSX_ERR_INVALID, "null pointer");
  if (nspecies <= 0 || oversample <= 0 || n0 < 2 || n1 < 2 || n0 % oversample || n1 % oversample)
    return fail(MSX_ERR_INVALID, "bad window grid %d x %d (oversample %d, %d species)", n0, n1, oversample, nspecies);
  if (!(potential_range > 0)) return fail(MSX_ERR_INVALID, "potential range must be positive");
  if ((size_t)(n0 / oversample) * (n1 / oversample) > (size_t)65535 * 128)
    return fail(MSX_ERR_INVALID, "window %d x %d too large", n0 / oversample, n1 / oversample);
  MSX_CUDA(launch_atom_windows(coeff_dev, nspecies, n0, n1, oversample, potential_range, windows_out_dev,
                               (cudaStream_t)stream), "atom windows");
  return MSX_OK;
}

int msx_build_transmission(const int* sites_dev, const int* slice_offsets_dev, int num_slices, const float* windows_dev,
                           int window_h, int window_w, int ny, int nx, float sigma, float* trans_out_dev,
                           float* potential_out_dev, void* stream) {
  if (num_slices < 0 || ny <= 0 || nx <= 0 || window_h <= 0 || window_w <= 0)
    return fail(MSX_ERR_INVALID, "bad sizes (slices %d, grid %d x %d, window %d x %d)", num_slices, ny, nx, window_h,
                window_w);
  if (num_slices == 0) return MSX_OK;
  if (!sites_dev || !slice_offsets_dev || !windows_dev || !trans_out_dev) return fail(MSX_ERR_INVALID, "null pointer");
  if (!aligned(sites_dev, 16)) return fail(MSX_ERR_INVALID, "sites must be 16-byte aligned (int32 rows of 4)");
  if (!aligned(trans_out_dev, 8)) return fail(MSX_ERR_INVALID, "transmission output must be 8-byte aligned");
  if (num_slices > 65535) return fail(MSX_ERR_INVALID, "at most 65535 slices");
  MSX_CUDA(launch_potential(reinterpret_cast<const int4*>(sites_dev), slice_offsets_dev, num_slices, windows_dev, window_h,
                            window_w, ny, nx, sigma, reinterpret_cast<float2*>(trans_out_dev), potential_out_dev,
                            (cudaStream_t)stream), "transmission slices");
  return MSX_OK;
}

int msx_build_probe(int ny, int nx, float kmax, double lambda, float k_semi, double c1, double c3, double c5,
                    int smooth_aperture, float* psi_k_out_dev, float* aperture_out_dev, double* normalization_dev,
                    void* stream) {
  if (ny < 2 || nx < 2 || ny > 65535) return fail(MSX_ERR_INVALID, "bad grid %d x %d", ny, nx);
  if (!psi_k_out_dev) return fail(MSX_ERR_INVALID, "null psi_k output");
  if (!aligned(psi_k_out_dev, 8)) return fail(MSX_ERR_INVALID, "psi_k must be 8-byte aligned");
  if (!(lambda > 0) || !(kmax > 0)) return fail(MSX_ERR_INVALID, "lambda and kmax must be positive");
  MSX_CUDA(launch_probe(ny, nx, kmax, lambda, k_semi, c1, c3, c5, smooth_aperture,
                        reinterpret_cast<float2*>(psi_k_out_dev), aperture_out_dev, normalization_dev,
                        (cudaStream_t)stream), "probe");
  return MSX_OK;
}

int msx_plan_create(int ny, int nx, int group, msx_plan** out) {
  if (!out) return fail(MSX_ERR_INVALID, "null plan pointer");
  *out = nullptr;
  if (!msx_supported_size(ny) || !msx_supported_size(nx))
    return fail(MSX_ERR_UNSUPPORTED, "grid %d x %d: supported line lengths are 64, 128, 256, 384, 512, 768, 1024", ny, nx);
  if (group < 0) return fail(MSX_ERR_INVALID, "group must be >= 0");
  int device = 0;
  MSX_CUDA(cudaGetDevice(&device), "cudaGetDevice");
  msx_plan* p = new msx_plan();
  p->ny = ny;
  p->nx = nx;
  p->device = device;
  int rc = msx_plan_set_schedule(p, default_row_schedule(nx), default_col_schedule(ny),
                                 group > 0 ? group : auto_group(ny, nx));
  if (rc == MSX_OK) {
    cudaError_t e = cudaMalloc(&p->ptab, sizeof(float2) * (size_t)ny * nx);
    if (e == cudaSuccess) e = cudaMalloc(&p->pyx, sizeof(float2) * (size_t)(ny + nx));
    if (e == cudaSuccess) e = cudaMalloc(&p->band, sizeof(int2) * (size_t)nx);
    if (e == cudaSuccess) e = cudaMalloc(&p->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->err, 0, sizeof(int));
    if (e != cudaSuccess) rc = fail(MSX_ERR_ALLOC, "plan table allocation failed");
  }
  if (rc == MSX_OK) {
    cudaError_t e = cudaStreamCreateWithFlags(&p->work, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming);
    if (e != cudaSuccess) rc = cuda_fail(e, "plan stream/events");
  }
  if (rc != MSX_OK) {
    msx_plan_destroy(p);
    return rc;
  }
  *out = p;
  return MSX_OK;
}

int msx_plan_destroy(msx_plan* p) {
  if (!p) return MSX_OK;
  drop_graph(p);
  if (p->psi) cudaFree(p->psi);
  if (p->ptab) cudaFree(p->ptab);
  if (p->pyx) cudaFree(p->pyx);
  if (p->band) cudaFree(p->band);
  if (p->err) cudaFree(p->err);
  if (p->partial) cudaFree(p->partial);
  if (p->inv_n) cudaFree(p->inv_n);
  if (p->tw_row) cudaFree(p->tw_row);
  if (p->tw_col) cudaFree(p->tw_col);
  for (void* q : {(void*)p->io_trans, (void*)p->io_psik, (void*)p->io_pos, (void*)p->io_norm, (void*)p->io_cbed})
    if (q) cudaFree(q);
  if (p->ev_copy) cudaEventDestroy(p->ev_copy);
  if (p->copy) cudaStreamDestroy(p->copy);
  if (p->ev_in) cudaEventDestroy(p->ev_in);
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  if (p->work) cudaStreamDestroy(p->work);
  delete p;
  return MSX_OK;
}

int msx_plan_set_schedule(msx_plan* p, int row_schedule, int col_schedule, int group) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  const SchedOps *rops, *cops;
  const int nr = schedule_table(p->nx, &rops), nc = schedule_table(p->ny, &cops);
  if (row_schedule < 0 || row_schedule >= nr || col_schedule < 0 || col_schedule >= nc)
    return fail(MSX_ERR_INVALID, "schedule (%d, %d) out of range (%d, %d)", row_schedule, col_schedule, nr, nc);
  if (group < 0 || group > 65535) return fail(MSX_ERR_INVALID, "group %d out of range", group);
  int rc = ensure_configured(p->device, p->nx, row_schedule, rops[row_schedule]);
  if (rc == MSX_OK) rc = ensure_configured(p->device, p->ny, col_schedule, cops[col_schedule]);
  if (rc != MSX_OK) return rc;
  if (!p->row_ops || p->row_sched != row_schedule) {
    rc = upload_twiddles(rops[row_schedule], &p->tw_row);
    if (rc != MSX_OK) return rc;
  }
  if (!p->col_ops || p->col_sched != col_schedule) {
    rc = upload_twiddles(cops[col_schedule], &p->tw_col);
    if (rc != MSX_OK) return rc;
  }
  p->row_sched = row_schedule;
  p->col_sched = col_schedule;
  p->row_ops = &rops[row_schedule];
  p->col_ops = &cops[col_schedule];
  const int old_group = p->group;
  if (group > 0) p->group = group;
  drop_graph(p);
  rc = ensure_workspace(p, (size_t)p->group);
  if (rc != MSX_OK) {
    // keep the previous group (and its workspace); the new schedule still applies
    const std::string msg = g_err;
    p->group = old_group;
    const int rc2 = (p->psi && (size_t)p->group <= p->psi_waves) ? prepare_tma(p) : MSX_OK;
    if (rc2 != MSX_OK) return rc2;
    g_err = msg;
    return MSX_ERR_ALLOC;
  }
  return prepare_tma(p);
}

int msx_plan_get_schedule(const msx_plan* p, int* row_schedule, int* col_schedule, int* group) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  if (row_schedule) *row_schedule = p->row_sched;
  if (col_schedule) *col_schedule = p->col_sched;
  if (group) *group = p->group;
  return MSX_OK;
}

int msx_plan_set_tma(msx_plan* p, int enable) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  p->use_tma = enable != 0;
  drop_graph(p);
  return MSX_OK;
}

int msx_plan_check(msx_plan* p) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  int h = 0;
  MSX_CUDA(cudaMemcpy(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost), "reading the plan error word");
  if (h) {
    MSX_CUDA(cudaMemset(p->err, 0, sizeof(int)), "clearing the plan error word");
    if (h & 2)  // bit 1: the paired row pass found its shared memory misaligned and did nothing
      return fail(MSX_ERR_CUDA, "the paired row pass found its shared memory misaligned (error word 0x%x)", h);
    return fail(MSX_ERR_TIMEOUT, "a pipelined pass gave up waiting for its tile copy (error word 0x%x)", h);
  }
  return MSX_OK;
}

int msx_plan_set_graph(msx_plan* p, int enable) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  p->use_graph = enable != 0;
  if (!p->use_graph) drop_graph(p);
  return MSX_OK;
}

int msx_multislice(msx_plan* p, const float* trans_dev, int num_slices, const float* psi_k_dev,
                   const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                   double lambda, double slice_t, float k_band, float* cbed_out_dev, int crop_y, int crop_x,
                   void* stream) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  if (num_probes < 0 || num_slices < 0) return fail(MSX_ERR_INVALID, "negative probe or slice count");
  if (num_probes == 0) return MSX_OK;
  if (crop_y <= 0 || crop_x <= 0 || crop_y > p->ny || crop_x > p->nx)
    return fail(MSX_ERR_INVALID, "crop %d x %d outside the %d x %d grid", crop_y, crop_x, p->ny, p->nx);
  if (!psi_k_dev || !normalization_dev || !positions_dev || !cbed_out_dev || (num_slices > 0 && !trans_dev))
    return fail(MSX_ERR_INVALID, "null pointer");
  if (!aligned(trans_dev, 8) || !aligned(psi_k_dev, 8) || !aligned(positions_dev, 8) || !aligned(normalization_dev, 8))
    return fail(MSX_ERR_INVALID, "complex inputs, positions and the normalisation must be 8-byte aligned");
  if (!(kmax > 0) || !(lambda > 0) || !(slice_t >= 0) || !(k_band >= 0))
    return fail(MSX_ERR_INVALID, "kmax, lambda must be positive; slice thickness and k_band non-negative");
  int dev = 0;
  MSX_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev != p->device) return fail(MSX_ERR_INVALID, "plan belongs to device %d, current device is %d", p->device, dev);

  MsArgs a;
  std::memset(&a, 0, sizeof(a));  // the struct doubles as the graph cache key: no stray padding bytes
  a.trans = trans_dev; a.num_slices = num_slices; a.psik = psi_k_dev; a.norm = normalization_dev;
  a.pos = positions_dev; a.num_probes = num_probes; a.kmax = kmax; a.lambda = lambda; a.slice_t = slice_t;
  a.k_band = k_band; a.cbed = cbed_out_dev; a.crop_y = crop_y; a.crop_x = crop_x;
  a.group = p->group; a.row_sched = p->row_sched; a.col_sched = p->col_sched;
  cudaStream_t caller = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MSX_CUDA(cudaStreamIsCapturing(caller, &cap), "cudaStreamIsCapturing");
  if (cap != cudaStreamCaptureStatusNone || !p->use_graph) return enqueue_multislice(p, a, caller);

  // Run on the plan's stream, ordered after and before the caller's stream.
  MSX_CUDA(cudaEventRecord(p->ev_in, caller), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(p->work, p->ev_in, 0), "cudaStreamWaitEvent");
  std::vector<unsigned char> key(sizeof(MsArgs));
  std::memcpy(key.data(), &a, sizeof(MsArgs));
  if (!p->gexec || key != p->gkey) {
    drop_graph(p);
    cudaGraph_t graph = nullptr;
    MSX_CUDA(cudaStreamBeginCapture(p->work, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    const int rc = enqueue_multislice(p, a, p->work);
    cudaError_t e = cudaStreamEndCapture(p->work, &graph);
    if (rc != MSX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&p->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      p->gexec = nullptr;
      return cuda_fail(e, "cudaGraphInstantiate");
    }
    p->gkey = key;
  }
  MSX_CUDA(cudaGraphLaunch(p->gexec, p->work), "cudaGraphLaunch");
  MSX_CUDA(cudaEventRecord(p->ev_out, p->work), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(caller, p->ev_out, 0), "cudaStreamWaitEvent");
  return MSX_OK;
}

int msx_multislice_detect(msx_plan* p, const float* trans_dev, int num_slices, const float* psi_k_dev,
                          const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                          double lambda, double slice_t, float k_band, const float* detectors_dev, int num_detectors,
                          float* signals_out_dev, void* stream) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  if (num_probes < 0 || num_slices < 1) return fail(MSX_ERR_INVALID, "detector mode needs num_slices >= 1");
  if (num_probes == 0) return MSX_OK;
  if (num_detectors < 1 || num_detectors > kMaxDetectors)
    return fail(MSX_ERR_INVALID, "1..%d detectors supported, got %d", kMaxDetectors, num_detectors);
  if (!trans_dev || !psi_k_dev || !normalization_dev || !positions_dev || !detectors_dev || !signals_out_dev)
    return fail(MSX_ERR_INVALID, "null pointer");
  if (!(kmax > 0) || !(lambda > 0) || !(slice_t >= 0) || !(k_band >= 0))
    return fail(MSX_ERR_INVALID, "kmax, lambda must be positive; slice thickness and k_band non-negative");
  const size_t need = (size_t)p->group * (p->nx / p->col_ops->col_c) * num_detectors;
  if (need > p->partial_words) {
    if (p->partial) cudaFree(p->partial);
  if (p->inv_n) cudaFree(p->inv_n);
    p->partial = nullptr;
    p->partial_words = 0;
    if (cudaMalloc(&p->partial, need * sizeof(float)) != cudaSuccess)
      return fail(MSX_ERR_ALLOC, "detector partial sums allocation failed");
    p->partial_words = need;
  }
  MsArgs a;
  std::memset(&a, 0, sizeof(a));
  a.trans = trans_dev; a.num_slices = num_slices; a.psik = psi_k_dev; a.norm = normalization_dev;
  a.pos = positions_dev; a.num_probes = num_probes; a.kmax = kmax; a.lambda = lambda; a.slice_t = slice_t;
  a.k_band = k_band; a.crop_y = p->ny; a.crop_x = p->nx; a.group = p->group; a.row_sched = p->row_sched;
  a.col_sched = p->col_sched; a.det = detectors_dev; a.ndet = num_detectors; a.signals = signals_out_dev;
  drop_graph(p);  // the detector sequence is launched directly
  return enqueue_multislice(p, a, (cudaStream_t)stream);
}

int msx_propagator_table(int ny, int nx, float kmax, double lambda, double slice_t, float k_band, float* ptab_out_dev,
                         void* stream) {
  if (ny < 2 || nx < 2 || ny > 65535 || !ptab_out_dev || !(kmax > 0) || !(lambda > 0) || !(slice_t >= 0))
    return fail(MSX_ERR_INVALID, "propagator table: bad arguments");
  MSX_CUDA(launch_ptab(ny, nx, kmax, lambda, slice_t, k_band, reinterpret_cast<float2*>(ptab_out_dev),
                       (cudaStream_t)stream), "propagator table");
  return MSX_OK;
}

int msx_plan_probe_waves(msx_plan* p, const float* psi_k_dev, const float* positions_dev, int num_probes, float kmax,
                         float* waves_out_dev, void* stream) {
  if (!p || num_probes < 0 || !psi_k_dev || !positions_dev || !waves_out_dev || !(kmax > 0))
    return fail(MSX_ERR_INVALID, "probe waves: bad arguments");
  if (num_probes == 0) return MSX_OK;
  cudaStream_t st = (cudaStream_t)stream;
  ColArgs c{};
  c.psi = reinterpret_cast<float2*>(waves_out_dev); c.psik = reinterpret_cast<const float2*>(psi_k_dev);
  c.pos_yx = positions_dev; c.tw = p->tw_col; c.G = num_probes; c.Nx = p->nx; c.kmax = kmax; c.x_begin = 0;
  c.ncols = p->nx;
  MSX_CUDA(p->col_ops->col(COL_INIT, c, st), "probe formation pass");
  MSX_CUDA(p->row_ops->row_mode(ROW_I, c.psi, nullptr, p->tw_row, num_probes, p->ny, st), "inverse row transform");
  return MSX_OK;
}

int msx_plan_probe_stack(msx_plan* p, const float* psi_k_dev, const double* normalization_dev,
                         const float* positions_dev, int num_probes, float kmax, float* probes_out_dev, void* stream) {
  if (!p || num_probes < 0 || !psi_k_dev || !normalization_dev || !positions_dev || !probes_out_dev || !(kmax > 0))
    return fail(MSX_ERR_INVALID, "probe stack: bad arguments");
  if (!aligned(psi_k_dev, 8) || !aligned(normalization_dev, 8) || !aligned(positions_dev, 8) ||
      !aligned(probes_out_dev, 8))
    return fail(MSX_ERR_INVALID, "probe stack: arrays must be 8-byte aligned");
  if (num_probes == 0) return MSX_OK;
  cudaStream_t st = (cudaStream_t)stream;
  ColArgs c{};
  c.psi = reinterpret_cast<float2*>(probes_out_dev); c.psik = reinterpret_cast<const float2*>(psi_k_dev);
  c.pos_yx = positions_dev; c.tw = p->tw_col; c.G = num_probes; c.Nx = p->nx; c.kmax = kmax; c.x_begin = 0;
  c.ncols = p->nx; c.init_norm = normalization_dev;
  MSX_CUDA(p->col_ops->col(COL_INIT, c, st), "probe formation pass");
  MSX_CUDA(p->row_ops->row_mode(ROW_I, c.psi, nullptr, p->tw_row, num_probes, p->ny, st), "inverse row transform");
  return MSX_OK;
}

int msx_plan_step_waves(msx_plan* p, float* waves_dev, int num_waves, const float* trans_dev, const float* ptab_dev,
                        void* stream) {
  if (!p || num_waves < 0 || !waves_dev || !trans_dev || !ptab_dev) return fail(MSX_ERR_INVALID, "step waves: bad arguments");
  if (num_waves == 0) return MSX_OK;
  cudaStream_t st = (cudaStream_t)stream;
  float2* w = reinterpret_cast<float2*>(waves_dev);
  ColArgs c{};
  c.psi = w; c.ptab = reinterpret_cast<const float2*>(ptab_dev); c.tw = p->tw_col; c.G = num_waves; c.Nx = p->nx;
  c.x_begin = 0; c.ncols = p->nx;
  MSX_CUDA(p->row_ops->row_mode(ROW_TF, w, reinterpret_cast<const float2*>(trans_dev), p->tw_row, num_waves, p->ny, st),
           "transmit + forward row transform");
  MSX_CUDA(p->col_ops->col(COL_MID, c, st), "column pass");
  MSX_CUDA(p->row_ops->row_mode(ROW_I, w, nullptr, p->tw_row, num_waves, p->ny, st), "inverse row transform");
  return MSX_OK;
}

int msx_plan_cbed_waves(msx_plan* p, float* waves_dev, int num_waves, const double* normalization_dev,
                        float* cbed_out_dev, int crop_y, int crop_x, void* stream) {
  if (!p || num_waves < 0 || !waves_dev || !normalization_dev || !cbed_out_dev || crop_y <= 0 || crop_x <= 0 ||
      crop_y > p->ny || crop_x > p->nx)
    return fail(MSX_ERR_INVALID, "cbed of waves: bad arguments");
  if (num_waves == 0) return MSX_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (!p->inv_n) {
    if (cudaMalloc(&p->inv_n, sizeof(float2) * (size_t)p->ny * p->nx) != cudaSuccess)
      return fail(MSX_ERR_ALLOC, "constant table allocation failed");
    // P = 1 everywhere, k_band beyond every |k|: launch_ptab with zero thickness gives (1/N, 0)
    MSX_CUDA(launch_ptab(p->ny, p->nx, 1.0f, 1.0, 0.0, 3.0e38f, p->inv_n, st), "constant table");
  }
  float2* w = reinterpret_cast<float2*>(waves_dev);
  MSX_CUDA(p->row_ops->row_mode(ROW_F, w, nullptr, p->tw_row, num_waves, p->ny, st), "forward row transform");
  ColArgs c{};
  c.psi = w; c.ptab = p->inv_n; c.tw = p->tw_col; c.norm = normalization_dev; c.cbed = cbed_out_dev; c.G = num_waves;
  c.Nx = p->nx; c.x_begin = p->nx / 2 - crop_x / 2; c.ncols = crop_x; c.y0 = p->ny / 2 - crop_y / 2; c.crop_y = crop_y;
  MSX_CUDA(p->col_ops->col(COL_FINAL, c, st), "final column pass");
  return MSX_OK;
}

int msx_multislice_host(msx_plan* p, const float* trans_host, int num_slices, const float* psi_k_host,
                        double normalization, const float* positions_host, int num_probes, float kmax, double lambda,
                        double slice_t, float k_band, float* cbed_host, int crop_y, int crop_x, void* stream) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  if (num_probes < 0 || num_slices < 0) return fail(MSX_ERR_INVALID, "negative probe or slice count");
  if (num_probes == 0) return MSX_OK;
  if (crop_y <= 0 || crop_x <= 0 || crop_y > p->ny || crop_x > p->nx)
    return fail(MSX_ERR_INVALID, "crop %d x %d outside the %d x %d grid", crop_y, crop_x, p->ny, p->nx);
  if (!psi_k_host || !positions_host || !cbed_host || (num_slices > 0 && !trans_host))
    return fail(MSX_ERR_INVALID, "null pointer");
  if (!(normalization > 0) || !(kmax > 0) || !(lambda > 0) || !(slice_t >= 0) || !(k_band >= 0))
    return fail(MSX_ERR_INVALID, "normalisation, kmax, lambda must be positive; slice thickness and k_band non-negative");
  int dev = 0;
  MSX_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev != p->device) return fail(MSX_ERR_INVALID, "plan belongs to device %d, current device is %d", p->device, dev);
  if (!p->copy) {
    MSX_CUDA(cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking), "copy stream");
    MSX_CUDA(cudaEventCreateWithFlags(&p->ev_copy, cudaEventDisableTiming), "cudaEventCreate");
  }
  const size_t wave = (size_t)p->ny * p->nx, pattern = (size_t)crop_y * crop_x;
  int rc = grow(&p->io_trans, &p->io_trans_words, wave * num_slices, "transmission slices");
  if (rc == MSX_OK) rc = grow(&p->io_psik, &p->io_psik_words, wave, "k-space probe");
  if (rc == MSX_OK) rc = grow(&p->io_pos, &p->io_pos_words, 2 * (size_t)num_probes, "positions");
  size_t one = p->io_norm ? 1 : 0;
  if (rc == MSX_OK) rc = grow(&p->io_norm, &one, 1, "normalisation");
  if (rc == MSX_OK) rc = grow(&p->io_cbed, &p->io_cbed_words, pattern * num_probes, "CBED stack");
  if (rc != MSX_OK) return rc;

  cudaStream_t caller = (cudaStream_t)stream, w = p->work, cp = p->copy;
  // The whole call is captured into a CUDA graph and replayed while its
  // arguments (host and device buffers included) repeat, when every host buffer
  // is page-locked: copies from pageable memory stay outside graphs.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MSX_CUDA(cudaStreamIsCapturing(caller, &cap), "cudaStreamIsCapturing");
  auto locked = [](const void* q) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return at.type == cudaMemoryTypeHost;
  };
  const bool graph = p->use_graph && cap == cudaStreamCaptureStatusNone && locked(psi_k_host) &&
                     locked(positions_host) && locked(cbed_host) && (num_slices == 0 || locked(trans_host));
  struct HostKey {
    const void *trans, *psik, *pos, *cbed, *d_trans, *d_psik, *d_pos, *d_norm, *d_cbed;
    double normalization, lambda, slice_t;
    float kmax, k_band;
    int num_slices, num_probes, crop_y, crop_x, group, row_sched, col_sched, tma;
  } hk;
  std::memset(&hk, 0, sizeof(hk));  // the struct is the cache key: no stray padding bytes
  hk.trans = trans_host; hk.psik = psi_k_host; hk.pos = positions_host; hk.cbed = cbed_host;
  hk.d_trans = p->io_trans; hk.d_psik = p->io_psik; hk.d_pos = p->io_pos; hk.d_norm = p->io_norm;
  hk.d_cbed = p->io_cbed; hk.normalization = normalization; hk.lambda = lambda; hk.slice_t = slice_t;
  hk.kmax = kmax; hk.k_band = k_band; hk.num_slices = num_slices; hk.num_probes = num_probes; hk.crop_y = crop_y;
  hk.crop_x = crop_x; hk.group = p->group; hk.row_sched = p->row_sched; hk.col_sched = p->col_sched;
  hk.tma = p->use_tma ? 1 : 0;
  std::vector<unsigned char> key(sizeof(hk));
  std::memcpy(key.data(), &hk, sizeof(hk));
  // everything here follows the caller's earlier work and this plan's earlier calls
  MSX_CUDA(cudaEventRecord(p->ev_in, caller), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(w, p->ev_in, 0), "cudaStreamWaitEvent");
  if (graph && p->gexec_host && key == p->gkey_host) {
    MSX_CUDA(cudaGraphLaunch(p->gexec_host, w), "cudaGraphLaunch");
    MSX_CUDA(cudaEventRecord(p->ev_out, w), "cudaEventRecord");
    MSX_CUDA(cudaStreamWaitEvent(caller, p->ev_out, 0), "cudaStreamWaitEvent");
    return MSX_OK;
  }
  if (graph) {
    if (p->gexec_host) cudaGraphExecDestroy(p->gexec_host);
    p->gexec_host = nullptr;
    p->gkey_host.clear();
    MSX_CUDA(cudaStreamBeginCapture(w, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  }
  const int chunk = 8;
  const int nchunks = (num_slices + chunk - 1) / chunk;
  const int ngroups = (num_probes + p->group - 1) / p->group;
  std::vector<cudaEvent_t> chunk_ev(nchunks + 1, nullptr), group_ev(ngroups, nullptr);
  auto release = [&]() {  // events still pending are released when they complete
    for (cudaEvent_t e : chunk_ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : group_ev) if (e) cudaEventDestroy(e);
  };
  // everything between the start and the end of a capture: any failure returns
  // through here, so that the capture is always ended
  auto run = [&]() -> int {
    for (auto& e : chunk_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(MSX_ERR_CUDA, "cudaEventCreate");
    for (auto& e : group_ev)
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(MSX_ERR_CUDA, "cudaEventCreate");
    // the copy stream forks from the work stream (joining the capture, if any)
    MSX_CUDA(cudaEventRecord(p->ev_out, w), "cudaEventRecord");
    MSX_CUDA(cudaStreamWaitEvent(cp, p->ev_out, 0), "cudaStreamWaitEvent");
    MSX_CUDA(cudaMemcpyAsync(p->io_psik, psi_k_host, sizeof(float2) * wave, cudaMemcpyHostToDevice, cp), "probe upload");
    MSX_CUDA(cudaMemcpyAsync(p->io_pos, positions_host, sizeof(float) * 2 * num_probes, cudaMemcpyHostToDevice, cp),
             "position upload");
    // by value through a launch argument: no host memory to keep alive, no staging
    MSX_CUDA(launch_store_double(p->io_norm, normalization, cp), "normalisation");
    MSX_CUDA(cudaEventRecord(chunk_ev[nchunks], cp), "cudaEventRecord");
    for (int i = 0; i < nchunks; ++i) {
      const int s0 = i * chunk, s1 = (s0 + chunk < num_slices) ? s0 + chunk : num_slices;
      MSX_CUDA(cudaMemcpyAsync(p->io_trans + (size_t)s0 * wave, trans_host + 2 * (size_t)s0 * wave,
                               sizeof(float2) * (size_t)(s1 - s0) * wave, cudaMemcpyHostToDevice, cp),
               "slice upload");
      MSX_CUDA(cudaEventRecord(chunk_ev[i], cp), "cudaEventRecord");
    }
    MSX_CUDA(cudaStreamWaitEvent(w, chunk_ev[nchunks], 0), "cudaStreamWaitEvent");
    MsArgs a;
    std::memset(&a, 0, sizeof(a));
    a.trans = reinterpret_cast<const float*>(p->io_trans); a.num_slices = num_slices;
    a.psik = reinterpret_cast<const float*>(p->io_psik); a.norm = p->io_norm; a.pos = p->io_pos;
    a.num_probes = num_probes; a.kmax = kmax; a.lambda = lambda; a.slice_t = slice_t; a.k_band = k_band;
    a.cbed = p->io_cbed; a.crop_y = crop_y; a.crop_x = crop_x;
    a.group = p->group; a.row_sched = p->row_sched; a.col_sched = p->col_sched;
    HostPipe hp{cp, chunk, &chunk_ev, &group_ev, cbed_host, pattern};
    int r = enqueue_multislice(p, a, w, &hp);
    if (r != MSX_OK) return r;
    // the copy stream joins back: the work stream (and through it the caller) waits for the downloads
    MSX_CUDA(cudaEventRecord(p->ev_copy, cp), "cudaEventRecord");
    MSX_CUDA(cudaStreamWaitEvent(w, p->ev_copy, 0), "cudaStreamWaitEvent");
    return MSX_OK;
  };
  rc = run();
  if (graph) {
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(w, &g);
    release();
    if (rc != MSX_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t e2 = cudaGraphInstantiate(&p->gexec_host, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) {
      p->gexec_host = nullptr;
      return cuda_fail(e2, "cudaGraphInstantiate");
    }
    p->gkey_host = key;
    MSX_CUDA(cudaGraphLaunch(p->gexec_host, w), "cudaGraphLaunch");
  } else {
    release();
  }
  if (rc != MSX_OK) return rc;
  MSX_CUDA(cudaEventRecord(p->ev_out, w), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(caller, p->ev_out, 0), "cudaStreamWaitEvent");
  return MSX_OK;
}

int msx_plan_profile(msx_plan* p, const float* trans_dev, int num_slices, const float* psi_k_dev,
                     const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                     double lambda, double slice_t, float k_band, int iters, float* ms_out, void* stream) {
  if (!p || !ms_out) return fail(MSX_ERR_INVALID, "null plan or output");
  if (iters <= 0 || num_slices <= 0 || num_probes <= 0 || !trans_dev || !psi_k_dev || !normalization_dev || !positions_dev)
    return fail(MSX_ERR_INVALID, "profile needs slices, probes, inputs and iters > 0");
  const int ny = p->ny, nx = p->nx;
  const int gn = num_probes < p->group ? num_probes : p->group;
  if (!workspace_holds(p, gn))
    return fail(MSX_ERR_ALLOC, "the plan's workspace does not hold %d waves (an earlier allocation failed)", gn);
  const size_t wave = (size_t)ny * nx;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t ev[4];
  for (auto& e : ev) MSX_CUDA(cudaEventCreate(&e), "cudaEventCreate");
  MSX_CUDA(launch_ptab(ny, nx, kmax, lambda, slice_t, k_band, p->ptab, st), "propagator table");
  MSX_CUDA(launch_pfac(ny, nx, kmax, lambda, slice_t, k_band, p->pyx, p->band, st), "propagator factors");
  ColArgs c{};
  c.psi = p->psi; c.ptab = p->ptab; c.psik = reinterpret_cast<const float2*>(psi_k_dev); c.pos_yx = positions_dev;
  c.tw = p->tw_col; c.norm = normalization_dev; c.cbed = nullptr; c.G = gn; c.Nx = nx; c.kmax = kmax;
  c.x_begin = 0; c.ncols = nx; c.y0 = 0; c.crop_y = 0;
  MSX_CUDA(p->col_ops->col(COL_INIT, c, st), "probe formation pass");
  float row_ms = 0, col_ms = 0;
  const float2* trans = reinterpret_cast<const float2*>(trans_dev);
  // the steady-state passes of multislice: the band-limited column range
  int bx_lo = 0, bx_hi = 0;
  band_columns(nx, kmax, k_band, p->col_ops->col_c, &bx_lo, &bx_hi);
  for (int i = 0; i < iters; ++i) {
    const int s = i % num_slices;
    MSX_CUDA(cudaEventRecord(ev[0], st), "cudaEventRecord");
    int rc = slice_passes(p, trans + (size_t)s * wave, gn, c, false, st, bx_lo, bx_hi);
    if (rc != MSX_OK) return rc;
    MSX_CUDA(cudaEventRecord(ev[1], st), "cudaEventRecord");
    if (p->use_tma && p->map_ok) {
      TmaPassArgs ta{};
      ta.psi = p->psi; ta.tw = p->tw_col; ta.pyx = p->pyx; ta.band = p->band; ta.err = p->err;
      ta.G = gn; ta.Ny = ny; ta.Nx = nx; ta.x_lo = bx_lo; ta.x_hi = bx_hi;
      MSX_CUDA(p->col_ops->col_tma(p->map, ta, p->col_ctas, st), "column pass");
    } else {
      MSX_CUDA(p->col_ops->col(COL_MID, c, st), "column pass");
    }
    MSX_CUDA(cudaEventRecord(ev[2], st), "cudaEventRecord");
    MSX_CUDA(cudaEventSynchronize(ev[2]), "cudaEventSynchronize");
    float a = 0, b = 0;
    MSX_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]), "cudaEventElapsedTime");
    MSX_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]), "cudaEventElapsedTime");
    row_ms += a;
    col_ms += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  ms_out[0] = row_ms / iters;
  ms_out[1] = col_ms / iters;
  ms_out[2] = (float)gn;
  return MSX_OK;
}

int msx_plan_autotune(msx_plan* p, const float* trans_dev, int num_slices, const float* psi_k_dev,
                      const double* normalization_dev, const float* positions_dev, int num_probes, float kmax,
                      double lambda, double slice_t, float k_band, int iters, size_t max_workspace_bytes,
                      float* best_ns_per_wave_slice, void* stream) {
  if (!p) return fail(MSX_ERR_INVALID, "null plan");
  if (iters <= 0 || num_slices <= 0 || num_probes <= 0 || !trans_dev || !psi_k_dev || !normalization_dev || !positions_dev)
    return fail(MSX_ERR_INVALID, "autotune needs slices, probes, inputs and iters > 0");
  const SchedOps *rops, *cops;
  const int nr = schedule_table(p->nx, &rops), nc = schedule_table(p->ny, &cops);
  const size_t wave_bytes = sizeof(float2) * (size_t)p->ny * p->nx;
  if (max_workspace_bytes == 0) max_workspace_bytes = (size_t)1 << 30;
  // candidate groups: resident sets of 8 MiB .. 1 GiB, and every probe at once
  std::vector<int> groups;
  for (size_t mb : {8, 16, 32, 48, 64, 128, 256, 512, 1024}) {
    size_t g = (mb << 20) / wave_bytes;
    if (g < 1) g = 1;
    if (g > (size_t)num_probes) g = (size_t)num_probes;
    if (g * wave_bytes > max_workspace_bytes) continue;
    if (groups.empty() || groups.back() != (int)g) groups.push_back((int)g);
  }
  if (groups.empty()) groups.push_back(1);
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  MSX_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
  MSX_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
  const float2* trans = reinterpret_cast<const float2*>(trans_dev);
  const size_t wave = (size_t)p->ny * p->nx;
  // The row and column passes only share the group size, so for every group the
  // best row schedule and the best column schedule are found separately.
  float best = 1e30f;
  int br = p->row_sched, bc = p->col_sched, bg = p->group;
  int rc = MSX_OK;
  auto time_loop = [&](bool row_pass, int g, float* ms) -> int {
    ColArgs c{};
    c.psi = p->psi; c.ptab = p->ptab; c.psik = reinterpret_cast<const float2*>(psi_k_dev); c.pos_yx = positions_dev;
    c.tw = p->tw_col; c.norm = normalization_dev; c.G = g; c.Nx = p->nx; c.kmax = kmax; c.x_begin = 0; c.ncols = p->nx;
    MSX_CUDA(p->col_ops->col(COL_INIT, c, st), "probe formation pass");
    int bx_lo = 0, bx_hi = 0;  // time the steady-state (band-limited) passes
    band_columns(p->nx, kmax, k_band, p->col_ops->col_c, &bx_lo, &bx_hi);
    for (int pass = 0; pass < 2; ++pass) {  // pass 0 warms caches and clocks
      MSX_CUDA(cudaEventRecord(e0, st), "cudaEventRecord");
      for (int i = 0; i < iters; ++i) {
        if (row_pass) {
          const int r2 = slice_passes(p, trans + (size_t)(i % num_slices) * wave, g, c, false, st, bx_lo, bx_hi);
          if (r2 != MSX_OK) return r2;
        } else if (p->use_tma && p->map_ok) {
          TmaPassArgs ta{};
          ta.psi = p->psi; ta.tw = p->tw_col; ta.pyx = p->pyx; ta.band = p->band; ta.err = p->err;
          ta.G = g; ta.Ny = p->ny; ta.Nx = p->nx; ta.x_lo = bx_lo; ta.x_hi = bx_hi;
          MSX_CUDA(p->col_ops->col_tma(p->map, ta, p->col_ctas, st), "column pass");
        } else {
          MSX_CUDA(p->col_ops->col(COL_MID, c, st), "column pass");
        }
      }
      MSX_CUDA(cudaEventRecord(e1, st), "cudaEventRecord");
    }
    MSX_CUDA(cudaEventSynchronize(e1), "cudaEventSynchronize");
    MSX_CUDA(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime");
    return MSX_OK;
  };
  for (int g : groups) {
    float best_row = 1e30f, best_col = 1e30f;
    int gr = 0, gc = 0;
    for (int r = 0; r < nr && rc == MSX_OK; ++r) {
      rc = msx_plan_set_schedule(p, r, 0, g);
      if (rc != MSX_OK) break;
      MSX_CUDA(launch_ptab(p->ny, p->nx, kmax, lambda, slice_t, k_band, p->ptab, st), "propagator table");
      MSX_CUDA(launch_pfac(p->ny, p->nx, kmax, lambda, slice_t, k_band, p->pyx, p->band, st), "propagator factors");
      float ms = 0;
      rc = time_loop(true, g, &ms);
      if (rc == MSX_OK && ms < best_row) { best_row = ms; gr = r; }
    }
    for (int cidx = 0; cidx < nc && rc == MSX_OK; ++cidx) {
      rc = msx_plan_set_schedule(p, gr, cidx, g);
      if (rc != MSX_OK) break;
      MSX_CUDA(launch_ptab(p->ny, p->nx, kmax, lambda, slice_t, k_band, p->ptab, st), "propagator table");
      MSX_CUDA(launch_pfac(p->ny, p->nx, kmax, lambda, slice_t, k_band, p->pyx, p->band, st), "propagator factors");
      float ms = 0;
      rc = time_loop(false, g, &ms);
      if (rc == MSX_OK && ms < best_col) { best_col = ms; gc = cidx; }
    }
    if (rc != MSX_OK) break;
    const float ns = (best_row + best_col) * 1e6f / ((float)iters * (float)g);
    if (ns < best) { best = ns; br = gr; bc = gc; bg = g; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != MSX_OK) return rc;
  rc = msx_plan_set_schedule(p, br, bc, bg);
  if (best_ns_per_wave_slice) *best_ns_per_wave_slice = best;
  return rc;
}

}  // extern "C"

// ============================================================================ uneven batches
// A batch runs many independent jobs (crystals of different grid size,
// thickness, voltage and probe count) as one CUDA graph: the jobs are spread
// over `branches` parallel streams inside the capture (longest first onto the
// least loaded branch), each branch owning one plan per grid size, so the GPU
// overlaps jobs of different shapes.  The graph is replayed while the job list
// repeats.
struct msx_batch {
  int branches = 4;
  int device = 0;
  std::vector<std::vector<std::pair<long long, msx_plan*>>> plans;  // per branch: (ny<<32|nx, plan)
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;  // fork/join events, 2 per branch
  cudaStream_t origin = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned char> gkey;
  std::vector<std::pair<long long, std::array<int, 3>>> sched;  // (ny<<32|nx) -> row, col, group
};

namespace {

msx_plan* batch_plan(msx_batch* b, int branch, int ny, int nx, int* rc) {
  const long long key = ((long long)ny << 32) | (unsigned)nx;
  for (auto& kv : b->plans[branch])
    if (kv.first == key) return kv.second;
  // Persistent passes amortise their start-up over large groups: up to 1 GiB
  // of waves per branch (the jobs of a branch run one after another).
  int group = (int)(((size_t)1 << 30) / (sizeof(float2) * (size_t)ny * nx));
  if (group < 2) group = 2;
  int r = 0, c = 0;
  bool tuned = false;  // schedules set for this grid (else the plan's defaults)
  for (auto& kv : b->sched)
    if (kv.first == key) {
      r = kv.second[0]; c = kv.second[1]; tuned = true;
      if (kv.second[2] > 0) group = kv.second[2];
    }
  msx_plan* p = nullptr;
  *rc = msx_plan_create(ny, nx, group, &p);
  if (*rc != MSX_OK) return nullptr;
  if (tuned) {
    *rc = msx_plan_set_schedule(p, r, c, group);
    if (*rc != MSX_OK) { msx_plan_destroy(p); return nullptr; }
  }
  b->plans[branch].push_back({key, p});
  return p;
}

}  // namespace

extern "C" {

int msx_batch_create(int branches, msx_batch** out) {
  if (!out) return fail(MSX_ERR_INVALID, "null batch pointer");
  *out = nullptr;
  if (branches < 0 || branches > 16) return fail(MSX_ERR_INVALID, "branches must be 0..16");
  msx_batch* b = new msx_batch();
  b->branches = branches ? branches : 4;
  cudaError_t e = cudaGetDevice(&b->device);
  b->plans.resize(b->branches);
  b->streams.resize(b->branches, nullptr);
  b->events.resize(2 * b->branches, nullptr);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  for (int i = 0; i < b->branches && e == cudaSuccess; ++i) e = cudaStreamCreateWithFlags(&b->streams[i], cudaStreamNonBlocking);
  for (auto& ev : b->events)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    msx_batch_destroy(b);
    return cuda_fail(e, "batch streams/events");
  }
  *out = b;
  return MSX_OK;
}

int msx_batch_destroy(msx_batch* b) {
  if (!b) return MSX_OK;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  for (auto& br : b->plans)
    for (auto& kv : br) msx_plan_destroy(kv.second);
  for (auto s : b->streams)
    if (s) cudaStreamDestroy(s);
  for (auto ev : b->events)
    if (ev) cudaEventDestroy(ev);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->ev_out) cudaEventDestroy(b->ev_out);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return MSX_OK;
}

int msx_batch_set_schedule(msx_batch* b, int ny, int nx, int row_schedule, int col_schedule, int group) {
  if (!b) return fail(MSX_ERR_INVALID, "null batch");
  if (!msx_supported_size(ny) || !msx_supported_size(nx)) return fail(MSX_ERR_UNSUPPORTED, "grid %d x %d", ny, nx);
  if (row_schedule < 0 || row_schedule >= msx_num_schedules(nx) || col_schedule < 0 ||
      col_schedule >= msx_num_schedules(ny) || group < 0)
    return fail(MSX_ERR_INVALID, "schedule (%d, %d, group %d) out of range", row_schedule, col_schedule, group);
  const long long key = ((long long)ny << 32) | (unsigned)nx;
  bool found = false;
  for (auto& kv : b->sched)
    if (kv.first == key) { kv.second = {row_schedule, col_schedule, group}; found = true; }
  if (!found) b->sched.push_back({key, {row_schedule, col_schedule, group}});
  for (auto& br : b->plans)
    for (auto& kv : br)
      if (kv.first == key) {
        const int rc = msx_plan_set_schedule(kv.second, row_schedule, col_schedule, group);
        if (rc != MSX_OK) return rc;
      }
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->gkey.clear();
  return MSX_OK;
}

int msx_batch_autotune(msx_batch* b, const msx_job* jobs, int njobs, int iters, void* stream) {
  if (!b || (!jobs && njobs > 0) || njobs < 0 || iters <= 0) return fail(MSX_ERR_INVALID, "bad batch autotune arguments");
  // one representative per grid: the job with the most positions (ties: the first)
  std::vector<int> rep;
  for (int i = 0; i < njobs; ++i) {
    const msx_job& j = jobs[i];
    if (j.num_slices <= 0 || j.num_probes <= 0) continue;
    bool seen = false;
    for (int& r : rep)
      if (jobs[r].ny == j.ny && jobs[r].nx == j.nx) {
        seen = true;
        if (j.num_probes > jobs[r].num_probes) r = i;
      }
    if (!seen) rep.push_back(i);
  }
  for (int r : rep) {
    const msx_job& j = jobs[r];
    msx_plan* p = nullptr;
    int rc = msx_plan_create(j.ny, j.nx, 0, &p);
    if (rc != MSX_OK) return rc;
    // the batch keeps at most 1 GiB of waves per plan and branch
    rc = msx_plan_autotune(p, j.trans_dev, j.num_slices, j.psi_k_dev, j.normalization_dev, j.positions_dev,
                           j.num_probes, j.kmax, j.lambda, j.slice_t, j.k_band, iters, (size_t)1 << 30, nullptr,
                           stream);
    int row = 0, col = 0, group = 0;
    if (rc == MSX_OK) rc = msx_plan_get_schedule(p, &row, &col, &group);
    msx_plan_destroy(p);
    if (rc == MSX_OK) rc = msx_batch_set_schedule(b, j.ny, j.nx, row, col, group);
    if (rc != MSX_OK) return rc;
  }
  return MSX_OK;
}

int msx_batch_run(msx_batch* b, const msx_job* jobs, int njobs, void* stream) {
  if (!b) return fail(MSX_ERR_INVALID, "null batch");
  if (njobs < 0 || (njobs > 0 && !jobs)) return fail(MSX_ERR_INVALID, "bad job list");
  if (njobs == 0) return MSX_OK;
  int dev = 0;
  MSX_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev != b->device) return fail(MSX_ERR_INVALID, "batch belongs to device %d, current device is %d", b->device, dev);
  for (int i = 0; i < njobs; ++i) {
    const msx_job& j = jobs[i];
    if (!msx_supported_size(j.ny) || !msx_supported_size(j.nx))
      return fail(MSX_ERR_UNSUPPORTED, "job %d: grid %d x %d", i, j.ny, j.nx);
    if (j.num_probes < 0 || j.num_slices < 0 || j.crop_y <= 0 || j.crop_x <= 0 || j.crop_y > j.ny || j.crop_x > j.nx)
      return fail(MSX_ERR_INVALID, "job %d: bad probe/slice count or crop", i);
    if (j.num_probes > 0 && (!j.psi_k_dev || !j.normalization_dev || !j.positions_dev || !j.cbed_out_dev ||
                             (j.num_slices > 0 && !j.trans_dev)))
      return fail(MSX_ERR_INVALID, "job %d: null pointer", i);
    if (!(j.kmax > 0) || !(j.lambda > 0) || !(j.slice_t >= 0) || !(j.k_band >= 0))
      return fail(MSX_ERR_INVALID, "job %d: kmax, lambda must be positive", i);
  }
  cudaStream_t caller = (cudaStream_t)stream;
  std::vector<unsigned char> key(sizeof(msx_job) * (size_t)njobs);
  std::memcpy(key.data(), jobs, key.size());
  if (!b->gexec || key != b->gkey) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
    b->gkey.clear();
    // longest job first onto the least loaded branch
    std::vector<int> order(njobs);
    for (int i = 0; i < njobs; ++i) order[i] = i;
    auto cost = [&](int i) {
      const msx_job& j = jobs[i];
      const double n = (double)j.ny * j.nx;
      return (double)j.num_probes * (j.num_slices + 1) * n * std::log2(n);
    };
    std::sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    std::vector<double> load(b->branches, 0.0);
    std::vector<std::vector<int>> assign(b->branches);
    for (int i : order) {
      int best = 0;
      for (int k = 1; k < b->branches; ++k)
        if (load[k] < load[best]) best = k;
      load[best] += cost(i);
      assign[best].push_back(i);
    }
    // plans are created (allocating) before the capture
    for (int k = 0; k < b->branches; ++k)
      for (int i : assign[k]) {
        int rc = MSX_OK;
        if (!batch_plan(b, k, jobs[i].ny, jobs[i].nx, &rc)) return rc;
      }
    cudaGraph_t graph = nullptr;
    MSX_CUDA(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    int rc = MSX_OK;
    for (int k = 0; k < b->branches && rc == MSX_OK; ++k) {
      cudaError_t e = cudaEventRecord(b->events[2 * k], b->origin);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(b->streams[k], b->events[2 * k], 0);
      if (e != cudaSuccess) rc = cuda_fail(e, "batch fork");
      for (int i : assign[k]) {
        if (rc != MSX_OK) break;
        const msx_job& j = jobs[i];
        if (j.num_probes == 0) continue;
        msx_plan* p = batch_plan(b, k, j.ny, j.nx, &rc);
        MsArgs a;
        std::memset(&a, 0, sizeof(a));
        a.trans = j.trans_dev; a.num_slices = j.num_slices; a.psik = j.psi_k_dev; a.norm = j.normalization_dev;
        a.pos = j.positions_dev; a.num_probes = j.num_probes; a.kmax = j.kmax; a.lambda = j.lambda;
        a.slice_t = j.slice_t; a.k_band = j.k_band; a.cbed = j.cbed_out_dev; a.crop_y = j.crop_y; a.crop_x = j.crop_x;
        a.group = p->group; a.row_sched = p->row_sched; a.col_sched = p->col_sched;
        rc = enqueue_multislice(p, a, b->streams[k]);
      }
      if (rc == MSX_OK) {
        e = cudaEventRecord(b->events[2 * k + 1], b->streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->origin, b->events[2 * k + 1], 0);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch join");
      }
    }
    cudaError_t e = cudaStreamEndCapture(b->origin, &graph);
    if (rc != MSX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      b->gexec = nullptr;
      return cuda_fail(e, "cudaGraphInstantiate");
    }
    b->gkey = key;
  }
  MSX_CUDA(cudaEventRecord(b->ev_in, caller), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(b->origin, b->ev_in, 0), "cudaStreamWaitEvent");
  MSX_CUDA(cudaGraphLaunch(b->gexec, b->origin), "cudaGraphLaunch");
  MSX_CUDA(cudaEventRecord(b->ev_out, b->origin), "cudaEventRecord");
  MSX_CUDA(cudaStreamWaitEvent(caller, b->ev_out, 0), "cudaStreamWaitEvent");
  return MSX_OK;
}

int msx_batch_check(msx_batch* b) {
  if (!b) return fail(MSX_ERR_INVALID, "null batch");
  for (auto& br : b->plans)
    for (auto& kv : br) {
      const int rc = msx_plan_check(kv.second);
      if (rc != MSX_OK) return rc;
    }
  return MSX_OK;
}

}  // extern "C"
