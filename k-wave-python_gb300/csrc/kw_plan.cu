// Host side of libkwave_gb300: plan objects, uploads, the launch sequence of
// one time step, and the extern "C" entry points declared in
// include/kwave_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kwave_gb300.h"
#include "kw_kernels.cuh"

#define KW_VERSION 100  // 0.1.0

static thread_local std::string g_err;

static int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

// Lets other translation units of the library report through kw_last_error().
int kw_internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return fail(e_ == cudaErrorMemoryAllocation ? KW_ERR_OOM : KW_ERR_CUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                         \
  } while (0)

static const int kThreads = 256;

struct HostSrc {
  bool set = false;
  int mode = 0;
  std::vector<long long> idx;
  std::vector<float> sig;  // (nrows, len) row-major as given
  int nrows = 0, len = 0;
};

struct kw_plan {
  kw_grid_desc g{};
  int D = 0;
  int N[3] = {1, 1, 1};
  long long ntot = 0;
  int L = 0, H = 0, Hp = 0, Mfft = 0, even = 0, nrows = 0, R = 1;
  long long spec_elems = 0;
  bool finalized = false;
  int t = 0;
  // staged host inputs
  std::vector<float> hfield[9];
  float hscalar[9] = {0};
  std::vector<float> htab[7][3];
  HostSrc hsrc[6];
  std::vector<long long> sens_idx;
  int record_mask = 0;
  int interp_npts = 0, interp_nc = 0;
  std::vector<int> interp_slot;
  std::vector<double> interp_w;
  // device
  std::vector<void*> allocs;
  float* d_u[3] = {nullptr, nullptr, nullptr};
  float* d_rho[3] = {nullptr, nullptr, nullptr};
  float* d_p = nullptr;
  float* d_rhosum = nullptr;
  float2* d_S[KW_NBUF] = {nullptr};
  float* d_field[9] = {nullptr};
  float* d_tab[7][3] = {{nullptr}};
  float2* d_tw_axis[3] = {nullptr, nullptr, nullptr};
  KwFftLen flen_axis[3];
  float2* d_tw_row = nullptr;
  float2* d_twpost = nullptr;
  KwFftLen flen_row;
  KwSrcDev src[6];
  int* d_sens_rowptr = nullptr;
  int4* d_sens_ent = nullptr;
  int nslots = 0;
  float* d_rec[7] = {nullptr};
  int nrec = 0;
  int* d_islot = nullptr;
  double* d_iw = nullptr;
  size_t smem_rows = 0, smem_axis_plain[3] = {0, 0, 0}, smem_axis_ops = 0;
  int T_axis[3] = {1, 1, 1};
  // register-FFT dispatch (power-of-two lengths 64..1024)
  bool generic_only = false;
  bool axis_reg[3] = {false, false, false};
  int axis_regP[3] = {0, 0, 0}, axis_regE[3] = {0, 0, 0};
  bool rows_reg = false;
  // persistent TMA axis passes
  void* tma = nullptr;
  bool tma_axis[3] = {false, false, false};
  bool rows_tma = false;  // velocity / power-law density stages through kw_rows_tma
  // kw_plan_derive_medium request
  int derive_what = 0;
  std::vector<float> halpha;
  double alpha_s = 0.0, alpha_y = 0.0;
  int derive_absorb = 0;
  int nsm = 0;
  int rows_regP = 0, rows_regE = 0, rows_R = 0, rows_RS = 0;
  // p0 smoothing on the device
  bool smooth = false, p0s_ready = false;
  std::vector<float> hwin;
  double wrad = 0.0;
  float* d_win = nullptr;
  float* d_p0s = nullptr;
  float* d_p0scale = nullptr;
  unsigned int* d_maxes = nullptr;
  // per-step flags passed to the row stages
  int srcp_on = 0, srcu_on[3] = {0, 0, 0}, rec_us = 0, init_r2c = 0;
  // grouping: when set, the generic passes of a step are recorded here
  // instead of launched (kw_batch folds them into grouped launches)
  struct LaunchRec {
    int kind;  // 0 generic rows, 1 generic axis pass, 2 another kernel
    RowsParams rp;
    AxisParams ap;
    int gx, gy, gz;
    size_t smem;
  };
  std::vector<LaunchRec>* rec_list = nullptr;
  // step graphs: one captured step per distinct launch sequence, replayed with
  // the step index read from d_tstep
  struct StepGraph {
    int key;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    long long nlaunch;
  };
  std::vector<StepGraph> graphs;
  bool use_graphs = true;
  // TMA passes launched as programmatic dependents (KWAVE_GB300_PDL=1).  Off by
  // default: at 256^3 the step took 1.083 ms with it against 1.054 ms without
  // (early CTAs of the next persistent pass land unevenly across SMs).
  bool pdl = false;
  bool capturing = false;
  int* d_tstep = nullptr;
  int tstep_val = -1;  // value d_tstep holds once the stream reaches the last enqueued work
  cudaStream_t cap_stream = nullptr;
  int radix_order = 0;  // schedule of the Stockham stages (kRadixOrders)
  // checkpoints of the carried state for the sound-speed gradient: slot s
  // holds u_i, rho_i and the spectrum of p after step s * ckpt_K
  int ckpt_K = 0;
  std::vector<float*> ckpt;
  std::vector<char> ckpt_ok;
  // failure-detection test of the bounded waits (kw_plan_set_wait_test)
  int wait_test = 0;
  // set by kw_plan_adjoint around its ST_ADJ_A / ST_ADJ_E launches
  const float* adj_fsum = nullptr;
  float* adj_gacc = nullptr;
  // launch accounting / timing
  long long launches = 0;
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, size_t>> ev_used;  // (class, index of start event)
  size_t ev_next = 0;
};

// TMA passes start their prologue while the previous kernel drains, except
// while every launch is bracketed by timing events.
static int pdl_ok(const kw_plan* p) { return p->pdl && !p->timing; }

// Bracket a launch with events when timing is on.
static int ev_begin(kw_plan* p, cudaStream_t st, size_t* slot) {
  if (!p->timing) return KW_OK;
  if (p->ev_next + 2 > p->ev_pool.size()) {
    for (int i = 0; i < 256; ++i) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      p->ev_pool.push_back(e);
    }
  }
  *slot = p->ev_next;
  p->ev_next += 2;
  CK(cudaEventRecord(p->ev_pool[*slot], st));
  return KW_OK;
}

static int ev_end(kw_plan* p, cudaStream_t st, int cls, size_t slot) {
  p->launches++;
  if (!p->timing) return KW_OK;
  CK(cudaEventRecord(p->ev_pool[slot + 1], st));
  p->ev_used.push_back({cls, slot});
  return KW_OK;
}

// Schedules of the run-time-length shared-memory FFTs.  Orders 0-2: the
// order in which the factors 4, 2, 3, 5, 7 of a length become Stockham
// stages.  Order 3: the two-level schedule (two passes of register DFTs,
// kw_fft.cuh: fft2_smem) for lengths n1 n2 with both factors register-DFT
// sizes, the Stockham order 0 for the others.  Every schedule computes the
// same DFT; they differ in shared-memory traffic, instruction count, bank
// conflicts and rounding (kw_batch_autotune_radix picks one by timing).
static const int kRadixOrders[3][5] = {{4, 2, 3, 5, 7}, {5, 3, 7, 4, 2}, {3, 4, 5, 2, 7}};
static const int kTwoLevelOrder = 3;

static bool factor_len(int n, KwFftLen& f, int order = 0) {
  f.n = n;
  f.nst = 0;
  int m = n;
  const int* rs = kRadixOrders[order == kTwoLevelOrder ? 0 : order];
  for (int i = 0; i < 5; ++i) {
    const int r = rs[i];
    while (m % r == 0 && m > 1) {
      if (f.nst >= KW_MAX_STAGES) return false;
      f.radix[f.nst++] = r;
      m /= r;
    }
  }
  kw_fft_len_finish(f);
  if (order == kTwoLevelOrder && m == 1) kw_fft_len_two_level(f);
  return m == 1;
}

template <typename T>
static int dalloc(kw_plan* p, T** out, size_t count) {
  void* ptr = nullptr;
  size_t bytes = count * sizeof(T);
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&ptr, bytes);
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? KW_ERR_OOM : KW_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                cudaGetErrorString(e));
  p->allocs.push_back(ptr);
  *out = static_cast<T*>(ptr);
  return KW_OK;
}

template <typename T>
static int upload(kw_plan* p, T** out, const T* host, size_t count) {
  int rc = dalloc(p, out, count);
  if (rc) return rc;
  if (count) CK(cudaMemcpy(*out, host, count * sizeof(T), cudaMemcpyHostToDevice));
  return KW_OK;
}

static std::vector<float2> twiddles(int n, int count) {
  std::vector<float2> w(count);
  for (int j = 0; j < count; ++j) {
    const double a = -2.0 * M_PI * (double)j / (double)n;
    w[j] = make_float2((float)cos(a), (float)sin(a));
  }
  return w;
}

extern "C" {

int32_t kw_version(void) { return KW_VERSION; }

const char* kw_last_error(void) { return g_err.c_str(); }

int32_t kw_device_query(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor, uint64_t* free_bytes) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, dev));
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  if (free_bytes) {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    *free_bytes = fr;
  }
  return KW_OK;
}

int32_t kw_plan_create(const kw_grid_desc* desc, kw_plan** out) {
  if (!desc || !out) return fail(KW_ERR_INVALID, "kw_plan_create: null argument");
  if (desc->ndim != 2 && desc->ndim != 3) return fail(KW_ERR_UNSUPPORTED, "only 2-D and 3-D grids are supported (ndim=%d)", desc->ndim);
  if (desc->Nt < 1) return fail(KW_ERR_INVALID, "Nt must be >= 1 (got %d)", desc->Nt);
  if (desc->record_start < 0 || desc->record_start >= desc->Nt)
    return fail(KW_ERR_INVALID, "record start %d outside [0, Nt)", desc->record_start);
  kw_plan* p = new kw_plan();
  p->g = *desc;
  p->D = desc->ndim;
  p->ntot = 1;
  for (int a = 0; a < p->D; ++a) {
    p->N[a] = desc->shape[a];
    if (p->N[a] < 2 || p->N[a] > 4096) {
      delete p;
      return fail(KW_ERR_UNSUPPORTED, "grid size %d along axis %d outside [2, 4096]", desc->shape[a], a);
    }
    p->ntot *= p->N[a];
  }
  p->L = p->N[p->D - 1];
  p->H = p->L / 2 + 1;
  p->Hp = (p->H + 1) & ~1;
  p->even = (p->L % 2) == 0;
  p->Mfft = p->even ? p->L / 2 : p->L;
  p->nrows = (int)(p->ntot / p->L);
  p->spec_elems = (long long)p->nrows * p->Hp;
  for (int a = 0; a < p->D - 1; ++a) {
    if (!factor_len(p->N[a], p->flen_axis[a])) {
      int n = p->N[a];
      delete p;
      return fail(KW_ERR_UNSUPPORTED, "FFT length %d (axis %d) has a prime factor above 7", n, a);
    }
  }
  if (!factor_len(p->Mfft, p->flen_row)) {
    int n = p->L;
    delete p;
    return fail(KW_ERR_UNSUPPORTED, "FFT length %d (last axis) has a prime factor above 7", n);
  }
  for (int i = 0; i < 9; ++i) p->hscalar[i] = 0.f;
  *out = p;
  return KW_OK;
}

int32_t kw_plan_set_field(kw_plan* p, int32_t field, const float* host, int64_t n, float scalar) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (field < 0 || field > KW_F_P0) return fail(KW_ERR_INVALID, "unknown field id %d", field);
  if (host && n > 0) {
    if (n != p->ntot) return fail(KW_ERR_INVALID, "field %d has %lld values, grid has %lld", field, (long long)n, p->ntot);
    p->hfield[field].assign(host, host + n);
  } else {
    p->hfield[field].clear();
  }
  p->hscalar[field] = scalar;
  return KW_OK;
}

int32_t kw_plan_update_p0(kw_plan* p, const float* host, int64_t n) {
  if (!p || !host) return fail(KW_ERR_INVALID, "kw_plan_update_p0: null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_update_p0 before kw_plan_finalize");
  if (p->hfield[KW_F_P0].empty() || !p->d_field[KW_F_P0])
    return fail(KW_ERR_STATE, "kw_plan_update_p0: the plan was finalized without a p0 grid");
  if (n != p->ntot) return fail(KW_ERR_INVALID, "p0 has %lld values, grid has %lld", (long long)n, p->ntot);
  CK(cudaDeviceSynchronize());
  p->hfield[KW_F_P0].assign(host, host + n);
  CK(cudaMemcpy(p->d_field[KW_F_P0], host, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  p->p0s_ready = false;  // smoothing (if on) runs again on the new p0
  return kw_plan_reset(p);
}

int32_t kw_plan_update_source(kw_plan* p, int32_t slot, const float* signal, int32_t n_rows, int32_t length) {
  if (!p || !signal) return fail(KW_ERR_INVALID, "kw_plan_update_source: null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_update_source before kw_plan_finalize");
  if (slot < 0 || slot > KW_S_U2 || !p->hsrc[slot].set || !p->src[slot].sig)
    return fail(KW_ERR_STATE, "kw_plan_update_source: source slot %d was not set before kw_plan_finalize", slot);
  HostSrc& h = p->hsrc[slot];
  if (n_rows != h.nrows || length != h.len)
    return fail(KW_ERR_INVALID, "kw_plan_update_source: signal is (%d, %d), the slot holds (%d, %d)", n_rows, length,
                h.nrows, h.len);
  CK(cudaDeviceSynchronize());
  h.sig.assign(signal, signal + (size_t)n_rows * length);
  std::vector<float> tm((size_t)length * n_rows);
  for (int r = 0; r < n_rows; ++r)
    for (int t = 0; t < length; ++t) tm[(size_t)t * n_rows + r] = signal[(size_t)r * length + t];
  CK(cudaMemcpy(const_cast<float*>(p->src[slot].sig), tm.data(), tm.size() * sizeof(float), cudaMemcpyHostToDevice));
  return KW_OK;
}

int32_t kw_plan_derive_medium(kw_plan* p, int32_t what, const float* alpha, int64_t n, double alpha_s, double alpha_power,
                              int32_t absorb_mode) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (what < 0 || what > 7) return fail(KW_ERR_INVALID, "derive_medium: bad selection %d", what);
  if ((what & 6) && absorb_mode != 1 && absorb_mode != 2) return fail(KW_ERR_INVALID, "derive_medium: absorb_mode %d", absorb_mode);
  if ((what & 4) && absorb_mode != 1) return fail(KW_ERR_INVALID, "derive_medium: eta needs the power law");
  if (alpha && n != p->ntot) return fail(KW_ERR_INVALID, "derive_medium: alpha has %lld values, grid has %lld", (long long)n, p->ntot);
  p->derive_what = what;
  if (alpha)
    p->halpha.assign(alpha, alpha + n);
  else
    p->halpha.clear();
  p->alpha_s = alpha_s;
  p->alpha_y = alpha_power;
  p->derive_absorb = absorb_mode;
  return KW_OK;
}

int32_t kw_plan_set_table(kw_plan* p, int32_t table, int32_t axis, const float* host, int64_t n_floats) {
  if (!p || !host) return fail(KW_ERR_INVALID, "null argument");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (table < 0 || table > KW_T_WCOORD || axis < 0 || axis >= p->D) return fail(KW_ERR_INVALID, "bad table %d / axis %d", table, axis);
  const bool cplx = table >= KW_T_OPGRAD && table <= KW_T_UNSTAG;
  const long long want = (long long)p->N[axis] * (cplx ? 2 : 1);
  if (n_floats != want) return fail(KW_ERR_INVALID, "table %d axis %d: %lld floats, expected %lld", table, axis, (long long)n_floats, want);
  p->htab[table][axis].assign(host, host + n_floats);
  return KW_OK;
}

int32_t kw_plan_set_p0_smoothing(kw_plan* p, const float* window, int32_t n, double radius) {
  if (!p || !window) return fail(KW_ERR_INVALID, "null argument");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (n < 2 || !(radius > 0.0)) return fail(KW_ERR_INVALID, "smoothing window needs n >= 2 and radius > 0");
  p->hwin.assign(window, window + n);
  p->wrad = radius;
  p->smooth = true;
  return KW_OK;
}

int32_t kw_plan_set_source(kw_plan* p, int32_t slot, int32_t mode, const int64_t* mask_index, int32_t n_points,
                           const float* signal, int32_t n_rows, int32_t length) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (slot < 0 || slot > KW_S_U2) return fail(KW_ERR_INVALID, "unknown source slot %d", slot);
  if ((slot % 3) >= p->D) return fail(KW_ERR_INVALID, "source slot %d beyond ndim", slot);
  if (mode < 0 || mode > KW_SRC_ADDITIVE_NC) return fail(KW_ERR_INVALID, "Unknown source mode: %d", mode);
  if (n_points <= 0 || !mask_index || !signal || length <= 0) return fail(KW_ERR_INVALID, "empty source");
  if (n_rows != 1 && n_rows != n_points)
    return fail(KW_ERR_INVALID, "source signal has %d rows for %d mask points", n_rows, n_points);
  HostSrc& s = p->hsrc[slot];
  s.set = true;
  s.mode = mode;
  s.idx.assign(mask_index, mask_index + n_points);
  for (long long v : s.idx)
    if (v < 0 || v >= p->ntot) return fail(KW_ERR_INVALID, "source index %lld outside grid", v);
  for (size_t i = 1; i < s.idx.size(); ++i)
    if (s.idx[i] <= s.idx[i - 1]) return fail(KW_ERR_INVALID, "source mask indices must be strictly increasing (C order)");
  s.sig.assign(signal, signal + (size_t)n_rows * length);
  s.nrows = n_rows;
  s.len = length;
  return KW_OK;
}

int32_t kw_plan_set_sensor(kw_plan* p, const int64_t* slot_index, int32_t n_slots, int32_t record_mask) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (n_slots < 0 || (n_slots > 0 && !slot_index)) return fail(KW_ERR_INVALID, "bad sensor slots");
  p->sens_idx.assign(slot_index, slot_index + n_slots);
  for (long long v : p->sens_idx)
    if (v < 0 || v >= p->ntot) return fail(KW_ERR_INVALID, "sensor index %lld outside grid", v);
  for (size_t i = 1; i < p->sens_idx.size(); ++i)
    if (p->sens_idx[i] <= p->sens_idx[i - 1]) return fail(KW_ERR_INVALID, "sensor slot indices must be strictly increasing");
  if (record_mask & ~0x7f) return fail(KW_ERR_INVALID, "bad record mask 0x%x", record_mask);
  for (int a = p->D; a < 3; ++a)
    if (record_mask & ((1 << (1 + a)) | (1 << (4 + a)))) return fail(KW_ERR_INVALID, "velocity record beyond ndim");
  p->record_mask = record_mask;
  return KW_OK;
}

int32_t kw_plan_set_sensor_interp(kw_plan* p, int32_t n_points, int32_t n_corners, const int32_t* slot,
                                  const double* weight) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  if (n_points <= 0 || n_corners <= 0 || !slot || !weight) return fail(KW_ERR_INVALID, "bad interpolation table");
  p->interp_npts = n_points;
  p->interp_nc = n_corners;
  p->interp_slot.assign(slot, slot + (size_t)n_points * n_corners);
  p->interp_w.assign(weight, weight + (size_t)n_points * n_corners);
  return KW_OK;
}

static int build_csr(kw_plan* p, const std::vector<long long>& idx, int** d_rowptr, int4** d_ent) {
  std::vector<int> rowptr(p->nrows + 1, 0);
  std::vector<int4> ent(idx.size());
  for (size_t i = 0; i < idx.size(); ++i) {
    const int row = (int)(idx[i] / p->L);
    const int pos = (int)(idx[i] % p->L);
    ent[i] = make_int4(row, pos, (int)i, 0);
    rowptr[row + 1]++;
  }
  for (int r = 0; r < p->nrows; ++r) rowptr[r + 1] += rowptr[r];
  int rc = upload(p, d_rowptr, rowptr.data(), rowptr.size());
  if (rc) return rc;
  return upload(p, d_ent, ent.data(), ent.size());
}

static int zero_state(kw_plan* p) {
  for (int a = 0; a < p->D; ++a) {
    CK(cudaMemset(p->d_u[a], 0, p->ntot * sizeof(float)));
    CK(cudaMemset(p->d_rho[a], 0, p->ntot * sizeof(float)));
  }
  CK(cudaMemset(p->d_p, 0, p->ntot * sizeof(float)));
  if (p->d_rhosum) CK(cudaMemset(p->d_rhosum, 0, p->ntot * sizeof(float)));
  for (int b = 0; b < KW_NBUF; ++b)
    if (p->d_S[b]) CK(cudaMemset(p->d_S[b], 0, p->spec_elems * sizeof(float2)));
  for (int s = 0; s < 7; ++s)
    if (p->d_rec[s]) CK(cudaMemset(p->d_rec[s], 0, (size_t)p->nrec * p->nslots * sizeof(float)));
  return KW_OK;
}

static void dfree_last(kw_plan* p, void* ptr);

static size_t rows_smem_bytes(const kw_plan* p, int R) {
  return sizeof(float2) * ((size_t)p->Mfft + p->L / 2 + 1 + 2 * (size_t)R * p->Mfft) +
         sizeof(float) * (size_t)KW_NREAL * R * p->L;
}

static int default_rows_per_block(const kw_plan* p) {
  const int R = (p->L >= 2048) ? 1 : 2048 / p->L;
  return R > 16 ? 16 : R;
}

// Launch geometry of the run-time-length kernels: R rows per row block and T
// columns per axis tile (a power of two).  0 selects the defaults: 2048 / L
// rows (at most 16) and 4 columns (one 32-byte sector per tile row; what the
// autotuner picked for batched 2-D events of 192..512 points) halved until a
// tile's buffers fit 100 KB.  Requested tiles are halved until they fit
// 200 KB.  The arithmetic of every row and column transform is the same for
// any R and T.
static void set_generic_geometry(kw_plan* p, int T_req, int R) {
  p->R = R > 0 ? R : default_rows_per_block(p);
  p->smem_rows = rows_smem_bytes(p, p->R);
  for (int a = 0; a < p->D - 1; ++a) {
    const int n = p->N[a];
    int T = T_req > 0 ? T_req : 4;
    const size_t cap = T_req > 0 ? 200 * 1024 : 100 * 1024;
    while (T > 1 && (size_t)3 * n * T * sizeof(float2) > cap) T /= 2;
    p->T_axis[a] = T;
    p->smem_axis_plain[a] = sizeof(float2) * ((size_t)n + 2 * (size_t)n * T);
    if (a == 0) p->smem_axis_ops = sizeof(float2) * ((size_t)n + 3 * (size_t)n * T);
  }
}

int32_t kw_plan_finalize(kw_plan* p) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (p->finalized) return fail(KW_ERR_STATE, "plan already finalized");
  const int D = p->D;
  int rc;
  // required tables
  for (int a = 0; a < D; ++a) {
    for (int tb : {KW_T_K, KW_T_PML, KW_T_PMLSG, KW_T_OPGRAD, KW_T_OPDIV})
      if (p->htab[tb][a].empty()) return fail(KW_ERR_INVALID, "table %d for axis %d not set", tb, a);
  }
  if (p->g.absorb_mode == 1 && !p->g.use_kspace && false) return KW_ERR_INVALID;
  // a k-space corrected pressure source is given once (slot P0, scaled without
  // 1/d_i); the per-component factor 1/d_i is applied on the device
  for (int sl = 1; sl < 3; ++sl)
    if (p->hsrc[sl].set && p->hsrc[KW_S_P0].set && p->hsrc[KW_S_P0].mode == KW_SRC_ADDITIVE)
      return fail(KW_ERR_INVALID, "a k-space corrected pressure source is set once, in slot KW_S_P0");

  // state and work buffers
  for (int a = 0; a < D; ++a) {
    if ((rc = dalloc(p, &p->d_u[a], p->ntot))) return rc;
    if ((rc = dalloc(p, &p->d_rho[a], p->ntot))) return rc;
  }
  if ((rc = dalloc(p, &p->d_p, p->ntot))) return rc;
  if (p->g.absorb_mode == 1)
    if ((rc = dalloc(p, &p->d_rhosum, p->ntot))) return rc;
  for (int b = 0; b < KW_NBUF; ++b) {
    bool need = b < D || b == B_P || (b < 2 && p->g.absorb_mode == 1);
    if (b == B_SRCP) need = p->hsrc[KW_S_P0].set && p->hsrc[KW_S_P0].mode == KW_SRC_ADDITIVE;
    if (b >= B_SRCU0 && b < B_SRCU0 + 3) {
      const HostSrc& h = p->hsrc[KW_S_U0 + (b - B_SRCU0)];
      need = (b - B_SRCU0) < D && h.set && h.mode == KW_SRC_ADDITIVE;
    }
    if (b >= B_US0 && b < B_US0 + 3) need = (b - B_US0) < D && (p->record_mask & (1 << (KW_R_UX + b - B_US0)));
    if (need && (rc = dalloc(p, &p->d_S[b], p->spec_elems))) return rc;
  }
  // medium fields
  for (int f = 0; f < 9; ++f)
    if (!p->hfield[f].empty())
      if ((rc = upload(p, &p->d_field[f], p->hfield[f].data(), p->hfield[f].size()))) return rc;
  if (p->derive_what) {
    DeriveParams Dp;
    memset(&Dp, 0, sizeof(Dp));
    Dp.ndim = D;
    for (int a = 0; a < 3; ++a) Dp.N[a] = a < D ? p->N[a] : 1;
    Dp.ntot = p->ntot;
    Dp.dt_f = (float)p->g.dt;
    Dp.use_sg = p->g.use_sg;
    Dp.rho0 = p->d_field[KW_F_RHO0];
    Dp.c0 = p->d_field[KW_F_C0];
    Dp.c0_s = p->hscalar[KW_F_C0];
    Dp.alpha_s = p->alpha_s;
    Dp.y = p->alpha_y;
    const double kPi = 3.14159265358979323846;
    Dp.db_fac = std::pow(1e-6 / (2.0 * kPi), p->alpha_y);
    Dp.db_fac_f = (float)Dp.db_fac;
    Dp.db_div = 20.0 * std::log10(std::exp(1.0));
    Dp.tan_fac = std::tan(kPi * p->alpha_y / 2.0);
    Dp.absorb = p->derive_absorb;
    float* dalpha = nullptr;
    if (!p->halpha.empty() && (rc = upload(p, &dalpha, p->halpha.data(), p->halpha.size()))) return rc;
    Dp.alpha = dalpha;
    if (p->derive_what & 1) {
      if (!Dp.rho0) return fail(KW_ERR_INVALID, "derive_medium: dt/rho0 needs a rho0 grid");
      for (int a = 0; a < D; ++a) {
        if (!p->d_field[KW_F_DTRSG0 + a] && (rc = dalloc(p, &p->d_field[KW_F_DTRSG0 + a], p->ntot))) return rc;
        Dp.dtrsg[a] = p->d_field[KW_F_DTRSG0 + a];
      }
    }
    if (p->derive_what & 2) {
      if (!p->d_field[KW_F_TAU] && (rc = dalloc(p, &p->d_field[KW_F_TAU], p->ntot))) return rc;
      Dp.tau = p->d_field[KW_F_TAU];
    }
    if (p->derive_what & 4) {
      if (!p->d_field[KW_F_ETA] && (rc = dalloc(p, &p->d_field[KW_F_ETA], p->ntot))) return rc;
      Dp.eta = p->d_field[KW_F_ETA];
    }
    const int grid = (int)std::min<long long>((p->ntot + 255) / 256, 4096);
    k_derive_medium<<<grid, 256>>>(Dp);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if (dalpha) dfree_last(p, dalpha);
  }
  // p0 smoothing
  if (p->smooth) {
    if (!p->d_field[KW_F_P0]) return fail(KW_ERR_INVALID, "p0 smoothing requested without a p0 grid");
    for (int a = 0; a < D; ++a)
      if (p->htab[KW_T_WCOORD][a].empty()) return fail(KW_ERR_INVALID, "smoothing coordinates for axis %d not set", a);
    if ((rc = upload(p, &p->d_win, p->hwin.data(), p->hwin.size()))) return rc;
    if ((rc = dalloc(p, &p->d_p0s, p->ntot))) return rc;
    if ((rc = dalloc(p, &p->d_p0scale, 1))) return rc;
    if ((rc = dalloc(p, &p->d_maxes, 2))) return rc;
  }
  // tables
  for (int tb = 0; tb < 7; ++tb)
    for (int a = 0; a < D; ++a)
      if (!p->htab[tb][a].empty())
        if ((rc = upload(p, &p->d_tab[tb][a], p->htab[tb][a].data(), p->htab[tb][a].size()))) return rc;
  // twiddles
  for (int a = 0; a < D - 1; ++a) {
    std::vector<float2> w = twiddles(p->N[a], p->N[a]);
    if ((rc = upload(p, &p->d_tw_axis[a], w.data(), w.size()))) return rc;
  }
  {
    std::vector<float2> w = twiddles(p->Mfft, p->Mfft);
    if ((rc = upload(p, &p->d_tw_row, w.data(), w.size()))) return rc;
    std::vector<float2> wp = twiddles(p->L, p->L / 2 + 1);
    if ((rc = upload(p, &p->d_twpost, wp.data(), wp.size()))) return rc;
  }
  // sources
  for (int sl = 0; sl < 6; ++sl) {
    KwSrcDev& s = p->src[sl];
    memset(&s, 0, sizeof(s));
    const HostSrc& h = p->hsrc[sl];
    if (!h.set) continue;
    s.active = 1;
    s.mode = h.mode;
    s.nsig = h.nrows;
    s.len = h.len;
    int* rp;
    int4* en;
    if ((rc = build_csr(p, h.idx, &rp, &en))) return rc;
    s.row_ptr = rp;
    s.ent = en;
    std::vector<float> tm((size_t)h.len * h.nrows);
    for (int r = 0; r < h.nrows; ++r)
      for (int t = 0; t < h.len; ++t) tm[(size_t)t * h.nrows + r] = h.sig[(size_t)r * h.len + t];
    float* ds;
    if ((rc = upload(p, &ds, tm.data(), tm.size()))) return rc;
    s.sig = ds;
  }
  // sensor
  p->nslots = (int)p->sens_idx.size();
  p->nrec = p->g.Nt - p->g.record_start;
  if (p->nslots > 0) {
    if ((rc = build_csr(p, p->sens_idx, &p->d_sens_rowptr, &p->d_sens_ent))) return rc;
    for (int s = 0; s < 7; ++s)
      if (p->record_mask & (1 << s)) {
        if ((rc = dalloc(p, &p->d_rec[s], (size_t)p->nrec * p->nslots))) return rc;
        CK(cudaMemset(p->d_rec[s], 0, (size_t)p->nrec * p->nslots * sizeof(float)));
      }
  }
  if (p->interp_npts > 0) {
    for (int v : p->interp_slot)
      if (v < 0 || v >= p->nslots) return fail(KW_ERR_INVALID, "interpolation slot %d outside [0, %d)", v, p->nslots);
    if ((rc = upload(p, &p->d_islot, p->interp_slot.data(), p->interp_slot.size()))) return rc;
    if ((rc = upload(p, &p->d_iw, p->interp_w.data(), p->interp_w.size()))) return rc;
  }
  if ((rc = zero_state(p))) return rc;

  // launch geometry
  set_generic_geometry(p, 0, 0);
  CK(kw_generic_attr_0(200 * 1024));
  CK(kw_generic_attr_1(200 * 1024));
  {
    const char* env = getenv("KWAVE_GB300_GENERIC_FFT");
    p->generic_only = (env && env[0] == '1') || (p->g.flags & KW_DESC_GENERIC_FFT);
  }
  {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  if (!p->generic_only) {
    const char* env = getenv("KWAVE_GB300_NO_TMA");
    const bool no_tma = env && env[0] == '1';
    // the TMA pass indexes a spectrum with 32-bit element offsets
    const bool fits32 = (long long)p->spec_elems < (1LL << 31);
    for (int a = 0; a < D - 1 && !no_tma && fits32; ++a) {
      if (!kw_tma_supported(p->N[a])) continue;
      if (!p->tma) p->tma = kw_tma_plan_create();
      int E, Pt;
      kw_reg_shape(p->N[a], &E, &Pt);
      // 2-D grids whose operator passes would leave SMs without a tile at
      // the normal tile width take the small tiles (KWAVE_GB300_SMALL_TILES=0: never)
      static const bool small_on = [] {
        const char* e = getenv("KWAVE_GB300_SMALL_TILES");
        return !(e && e[0] == '0');
      }();
      const bool small = small_on && D == 2 && kw_tma_small_wanted(p->N[0], p->Hp, p->nsm);
      kw_tma_set_small(p->tma, 0, small);
      bool ok = true;
      for (int b = 0; b < KW_NBUF; ++b) {
        if (!p->d_S[b]) continue;
        if (D == 3 && a == 0)
          ok &= kw_tma_encode(p->tma, 0, b, p->d_S[b], p->N[1] * p->Hp, p->N[0], (long long)p->N[1] * p->Hp, 1, 0, Pt);
        else if (D == 3)
          ok &= kw_tma_encode(p->tma, 1, b, p->d_S[b], p->Hp, p->N[1], p->Hp, p->N[0], (long long)p->N[1] * p->Hp, Pt);
        else
          ok &= kw_tma_encode(p->tma, 0, b, p->d_S[b], p->Hp, p->N[0], p->Hp, 1, 0, Pt);
      }
      if (ok) {
        CK(kw_tma_attr(p->N[a], D == 3 ? a : 0, small));
        p->tma_axis[a] = true;
      }
    }
    for (int a = 0; a < D - 1; ++a) {
      p->axis_reg[a] = kw_reg_shape(p->N[a], &p->axis_regE[a], &p->axis_regP[a]);
      if (p->axis_reg[a]) CK(kw_axis_reg_attr(p->N[a]));
    }
    if (p->even) {
      // the register row kernels index pairs with 32 bits
      p->rows_reg = p->ntot < (1LL << 32) && kw_reg_shape(p->Mfft, &p->rows_regE, &p->rows_regP);
      if (p->rows_reg) {
        p->rows_R = 128 / p->rows_regP;
        const int target = p->rows_regP == 4 ? 4 : (p->rows_regP == 8 ? 8 : 0);
        int rs = p->Mfft + p->rows_regE;
        while (rs % 16 != target) ++rs;
        p->rows_RS = rs;
        CK(kw_rows_v2_attr(p->Mfft));
        const char* env = getenv("KWAVE_GB300_ROWS_TMA");
        if (!(env && env[0] == '0') && kw_device_error_ptr()) {
          CK(kw_rows_tma_attr(p->Mfft, p->Hp, p->rows_RS));
          p->rows_tma = true;
        }
      }
    }
  }
  if ((rc = dalloc(p, &p->d_tstep, 1))) return rc;
  {
    const char* env = getenv("KWAVE_GB300_GRAPHS");
    if (env && env[0] == '0') p->use_graphs = false;
    env = getenv("KWAVE_GB300_PDL");
    if (env && env[0] == '1') p->pdl = true;
  }
  CK(cudaDeviceSynchronize());
  p->finalized = true;
  p->t = 0;
  return KW_OK;
}

// ---------------------------------------------------------------------------
// launch sequence
// ---------------------------------------------------------------------------
static void fill_rows(const kw_plan* p, RowsParams& P) {
  memset(&P, 0, sizeof(P));
  P.ndim = p->D;
  P.N0 = p->N[0];
  P.N1 = p->D == 3 ? p->N[1] : 1;
  P.L = p->L;
  P.H = p->H;
  P.Hp = p->Hp;
  P.Mfft = p->Mfft;
  P.even = p->even;
  P.nrows = p->nrows;
  P.R = p->R;
  P.dM = kw_divu_make((uint32_t)p->Mfft);
  P.dL = kw_divu_make((uint32_t)p->L);
  P.dH = kw_divu_make((uint32_t)p->H);
  for (int b = 0; b < KW_NBUF; ++b) P.S[b] = p->d_S[b];
  for (int a = 0; a < 3; ++a) {
    P.inv_d[a] = a < p->D ? (float)(1.0 / p->g.spacing[a]) : 0.f;
    P.u[a] = p->d_u[a];
    P.rho[a] = p->d_rho[a];
    P.pml[a] = p->d_tab[KW_T_PML][a];
    P.pmlsg[a] = p->d_tab[KW_T_PMLSG][a];
    P.dtrsg[a] = p->d_field[KW_F_DTRSG0 + a];
    P.dtrsg_s[a] = p->hscalar[KW_F_DTRSG0 + a];
  }
  P.p = p->d_p;
  P.rho_sum = p->d_rhosum;
  P.p0 = p->smooth ? p->d_p0s : p->d_field[KW_F_P0];
  P.p0w = p->d_p0s;
  P.p0_scale = p->smooth ? p->d_p0scale : nullptr;
  P.c0 = p->d_field[KW_F_C0];
  P.c0_s = p->hscalar[KW_F_C0];
  P.rho0 = p->d_field[KW_F_RHO0];
  P.rho0_s = p->hscalar[KW_F_RHO0];
  P.bona = p->d_field[KW_F_BONA];
  P.bona_s = p->hscalar[KW_F_BONA];
  P.tau = p->d_field[KW_F_TAU];
  P.tau_s = p->hscalar[KW_F_TAU];
  P.eta = p->d_field[KW_F_ETA];
  P.eta_s = p->hscalar[KW_F_ETA];
  P.absorb = p->g.absorb_mode;
  P.disp = p->g.dispersion;
  P.nonlin = p->g.nonlinear;
  P.dt = (float)p->g.dt;
  P.tw = p->d_tw_row;
  P.twpost = p->d_twpost;
  P.flen = p->flen_row;
  for (int s = 0; s < 6; ++s) P.src[s] = p->src[s];
  P.sens_row_ptr = p->d_sens_rowptr;
  P.sens_ent = p->d_sens_ent;
  P.nslots = p->nslots;
  for (int s = 0; s < 7; ++s) P.rec[s] = p->d_rec[s];
  P.fsum = p->adj_fsum;
  P.gacc = p->adj_gacc;
}

// Host-side checks that every buffer a launch will touch exists: an internal
// inconsistency becomes an error return instead of a device fault.
static int need_buf(const kw_plan* p, int b, const char* what) {
  if (b < 0 || b >= KW_NBUF || !p->d_S[b]) return fail(KW_ERR_STATE, "internal: spectrum %d (%s) not allocated", b, what);
  return KW_OK;
}

static int check_rows(const kw_plan* p, int stage, int init) {
  int rc;
  const int D = p->D;
  if ((stage == ST_INIT || stage == ST_P0FFT || stage == ST_P0BACK) && (rc = need_buf(p, B_P, "p"))) return rc;
  if ((stage == ST_P0FFT || stage == ST_P0BACK) && !p->d_p0s) return fail(KW_ERR_STATE, "internal: no smoothing buffer");
  if (stage == ST_U || stage == ST_RHO)
    for (int a = 0; a < D; ++a)
      if ((rc = need_buf(p, a, "work"))) return rc;
  if (stage == ST_U && !init)
    for (int a = 0; a < D; ++a)
      if (p->srcu_on[a] && (rc = need_buf(p, B_SRCU0 + a, "velocity source"))) return rc;
  if ((stage == ST_RHO || stage == ST_SRC) && p->srcp_on && (rc = need_buf(p, B_SRCP, "pressure source"))) return rc;
  if (stage == ST_SRC)
    for (int a = 0; a < D; ++a)
      if (p->srcu_on[a] && (rc = need_buf(p, B_SRCU0 + a, "velocity source"))) return rc;
  if (stage == ST_RHO || stage == ST_UREC)
    for (int a = 0; a < D; ++a)
      if (((p->rec_us >> a) & 1) && (rc = need_buf(p, B_US0 + a, "unstaggered velocity"))) return rc;
  if (stage == ST_RHO || stage == ST_EOS) {
    if ((rc = need_buf(p, B_P, "p"))) return rc;
    if (p->g.absorb_mode == 1 && !p->d_rhosum) return fail(KW_ERR_STATE, "internal: density sum not allocated");
  }
  if ((p->rec_us || stage == ST_UREC) && p->nslots == 0) return fail(KW_ERR_STATE, "internal: no sensor slots");
  if (stage >= ST_ADJ_A) {
    for (int a = 0; a < D; ++a)
      if ((rc = need_buf(p, a, "adjoint work"))) return rc;
    if ((stage == ST_ADJ_A || stage == ST_ADJ_D) && (!p->d_rec[KW_R_P] || p->nslots == 0 || !p->d_sens_rowptr))
      return fail(KW_ERR_STATE, "internal: adjoint stage without a residual buffer");
  }
  return KW_OK;
}

// Timing class of a row-stage launch (KW_K_NCLASS classes; the stages other
// than U, RHO and EOS count with INIT).
static int rows_class(int stage) {
  switch (stage) {
    case ST_U: return KW_K_ROWS_U;
    case ST_RHO:
    case ST_RHO_PL: return KW_K_ROWS_RHO;
    case ST_EOS: return KW_K_ROWS_EOS;
    default: return KW_K_ROWS_INIT;
  }
}

// The adjoint stages run on the register row kernels where the plan's rows
// do (KWAVE_GB300_ADJ_GENERIC=1: on the generic row kernels).
static bool adjoint_rows_reg() {
  static const bool on = [] {
    const char* e = getenv("KWAVE_GB300_ADJ_GENERIC");
    return !(e && e[0] == '1');
  }();
  return on;
}

static int launch_rows(kw_plan* p, int stage, int init, int t, int write_p, cudaStream_t st) {
  int crc = check_rows(p, stage, init);
  if (crc) return crc;
  RowsParams P;
  fill_rows(p, P);
  P.stage = stage;
  P.init = init;
  P.t = t;
  P.rec_row = (t >= p->g.record_start) ? t - p->g.record_start : -1;
  if (p->capturing) {
    // replayed for other steps: the step index comes from the device counter
    P.tdev = p->d_tstep;
    P.t = 0;
    P.rec_row = (t >= p->g.record_start) ? -p->g.record_start : -(1 << 30);
  }
  P.write_p = write_p;
  P.srcp_on = p->srcp_on;
  for (int a = 0; a < 3; ++a) P.srcu_on[a] = p->srcu_on[a];
  P.rec_us = p->rec_us;
  P.init_r2c = p->init_r2c;
  if (p->rec_list) {
    kw_plan::LaunchRec r{};
    r.kind = (p->rows_reg && (stage < ST_ADJ_A || adjoint_rows_reg())) ? 2 : 0;
    r.rp = P;
    r.gx = (p->nrows + p->R - 1) / p->R;
    r.gy = r.gz = 1;
    r.smem = p->smem_rows;
    p->rec_list->push_back(r);
    return KW_OK;
  }
  size_t slot = 0;
  int rc = ev_begin(p, st, &slot);
  if (rc) return rc;
  if (p->rows_reg && (stage < ST_ADJ_A || adjoint_rows_reg())) {
    P.R = p->rows_R;
    P.ex_stride = p->rows_RS;
    // the power-law density stage keeps the divergence in shared memory (one
    // float2 per thread and register pair)
    const bool dsm = stage == ST_RHO && p->g.absorb_mode == 1 && p->d_rhosum;
    const bool extra = P.srcp_on || P.srcu_on[0] || P.srcu_on[1] || P.srcu_on[2] || P.rec_us;
    if (stage == ST_U && !init && !extra && p->rows_tma) {
      if (p->wait_test) {
        P.withhold = 1;
        P.wait_ns = 20000000ull;  // 20 ms
      }
      CK(kw_rows_tma_launch(p->Mfft, ST_U, p->nsm, st, P, kw_device_error_ptr(), pdl_ok(p)));
    }
    else if (stage == ST_RHO && dsm && !extra && p->rows_tma)
      CK(kw_rows_tma_launch(p->Mfft, ST_RHO_PL, p->nsm, st, P, kw_device_error_ptr(), pdl_ok(p)));
    else if (stage == ST_EOS && p->rows_tma)
      CK(kw_rows_tma_launch(p->Mfft, ST_EOS, p->nsm, st, P, kw_device_error_ptr(), pdl_ok(p)));
    else {
      const size_t smem = sizeof(float2) * (2 * (size_t)p->Mfft + 1 + (size_t)p->rows_R * p->rows_RS +
                                            (dsm ? (size_t)128 * p->rows_regE : 0));
      CK(kw_rows_v2_launch(p->Mfft, stage, dim3((p->nrows + p->rows_R - 1) / p->rows_R), smem, st, P));
    }
  } else {
    const int grid = (p->nrows + p->R - 1) / p->R;
    CK(P.flen.n1 ? kw_rows_launch_1(dim3(grid), p->smem_rows, st, P) : kw_rows_launch_0(dim3(grid), p->smem_rows, st, P));
  }
  CK(cudaGetLastError());
  return ev_end(p, st, rows_class(stage), slot);
}

static void fill_axis_geom(const kw_plan* p, int axis, AxisParams& A) {
  memset(&A, 0, sizeof(A));
  for (int b = 0; b < KW_NBUF; ++b) A.bufs[b] = p->d_S[b];
  A.n = p->N[axis];
  A.flen = p->flen_axis[axis];
  A.tw = p->d_tw_axis[axis];
  A.T = p->T_axis[axis];
  A.ndim = p->D;
  A.H = p->H;
  A.Hp = p->Hp;
  if (p->D == 3) {
    if (axis == 0) {
      A.xs = (long long)p->N[1] * p->Hp;
      A.os = 0;
      A.ncols = p->N[1] * p->Hp;
    } else {
      A.xs = p->Hp;
      A.os = (long long)p->N[1] * p->Hp;
      A.ncols = p->Hp;
    }
  } else {
    A.xs = p->Hp;
    A.os = 0;
    A.ncols = p->Hp;
  }
}

static int launch_axis_plain(kw_plan* p, int axis, int inv, const int* bufs, int nb, cudaStream_t st) {
  for (int i = 0; i < nb; ++i) {
    int rc = need_buf(p, bufs[i], "plain pass");
    if (rc) return rc;
  }
  AxisParams A;
  fill_axis_geom(p, axis, A);
  A.mode = inv ? 1 : 0;
  for (int i = 0; i < nb; ++i) A.plain[i] = bufs[i];
  const int nouter = (p->D == 3 && axis == 1) ? p->N[0] : 1;
  if (p->rec_list) {
    kw_plan::LaunchRec r{};
    r.kind = (p->tma_axis[axis] || p->axis_reg[axis]) ? 2 : 1;
    r.ap = A;
    r.gx = (A.ncols + A.T - 1) / A.T;
    r.gy = nouter;
    r.gz = nb;
    r.smem = p->smem_axis_plain[axis];
    p->rec_list->push_back(r);
    return KW_OK;
  }
  size_t slot = 0;
  int rc = ev_begin(p, st, &slot);
  if (rc) return rc;
  if (p->tma_axis[axis]) {
    CK(kw_tma_launch(p->tma, axis, p->N[axis], nouter, nb, p->nsm, st, A, pdl_ok(p)));
  } else if (p->axis_reg[axis]) {
    const int E = p->axis_regE[axis], Pt = p->axis_regP[axis], T = 256 / Pt, n = p->N[axis];
    dim3 grid((A.ncols + T - 1) / T, nouter, nb);
    CK(kw_axis_reg_launch(n, grid, sizeof(float2) * ((size_t)n + (size_t)T * (n + E + 1)), st, A));
  } else {
    dim3 grid((A.ncols + A.T - 1) / A.T, nouter, nb);
    CK(A.flen.n1 ? kw_axis_launch_1(grid, p->smem_axis_plain[axis], st, A)
                 : kw_axis_launch_0(grid, p->smem_axis_plain[axis], st, A));
  }
  CK(cudaGetLastError());
  return ev_end(p, st, KW_K_AXIS_PLAIN, slot);
}

static int launch_axis_ops(kw_plan* p, const AxisJob* jobs, int nj, cudaStream_t st) {
  if (nj < 1 || nj > KW_MAX_JOBS) return fail(KW_ERR_STATE, "internal: %d operator jobs", nj);
  for (int i = 0; i < nj; ++i) {
    int rc = need_buf(p, jobs[i].in, "operator input");
    if (!rc) rc = need_buf(p, jobs[i].out, "operator output");
    if (rc) return rc;
    if (jobs[i].axis < 0 || jobs[i].axis >= p->D) return fail(KW_ERR_STATE, "internal: job axis %d", jobs[i].axis);
    const int tb = jobs[i].op == OP_GRAD ? KW_T_OPGRAD : jobs[i].op == OP_DIV ? KW_T_OPDIV
                 : jobs[i].op == OP_UNSTAG ? KW_T_UNSTAG : -1;
    if (tb >= 0 && !p->d_tab[tb][jobs[i].axis]) return fail(KW_ERR_STATE, "internal: operator table %d missing", tb);
    if (jobs[i].op == OP_WIN && (!p->d_win || !p->d_tab[KW_T_WCOORD][0])) return fail(KW_ERR_STATE, "internal: no window");
  }
  AxisParams A;
  fill_axis_geom(p, 0, A);
  A.mode = 2;
  A.njobs = nj;
  for (int i = 0; i < nj; ++i) A.jobs[i] = jobs[i];
  for (int a = 0; a < p->D; ++a) {
    A.k[a] = p->d_tab[KW_T_K][a];
    A.fg[a] = reinterpret_cast<const float2*>(p->d_tab[KW_T_OPGRAD][a]);
    A.fd[a] = reinterpret_cast<const float2*>(p->d_tab[KW_T_OPDIV][a]);
    A.us[a] = reinterpret_cast<const float2*>(p->d_tab[KW_T_UNSTAG][a]);
  }
  for (int a = 0; a < p->D; ++a) A.wc[a] = p->d_tab[KW_T_WCOORD][a];
  A.wtab = p->d_win;
  A.wlen = (int)p->hwin.size();
  A.wrad = (float)p->wrad;
  A.kcoef = (float)(p->g.c_ref * p->g.dt / 2.0);
  A.use_kspace = p->g.use_kspace;
  A.pow1 = (float)(p->g.alpha_power - 2.0);
  A.pow2 = (float)(p->g.alpha_power - 1.0);
  A.scale = (float)(1.0 / (double)p->ntot);
  if (p->rec_list) {
    kw_plan::LaunchRec r{};
    r.kind = (p->tma_axis[0] || p->axis_reg[0]) ? 2 : 1;
    r.ap = A;
    r.gx = (A.ncols + A.T - 1) / A.T;
    r.gy = r.gz = 1;
    r.smem = p->smem_axis_ops;
    p->rec_list->push_back(r);
    return KW_OK;
  }
  size_t slot = 0;
  int rc = ev_begin(p, st, &slot);
  if (rc) return rc;
  if (p->tma_axis[0]) {
    CK(kw_tma_launch(p->tma, 0, p->N[0], 1, 0, p->nsm, st, A, pdl_ok(p)));
  } else if (p->axis_reg[0]) {
    const int E = p->axis_regE[0], Pt = p->axis_regP[0], T = 256 / Pt, n = p->N[0];
    dim3 grid((A.ncols + T - 1) / T, 1, 1);
    CK(kw_axis_reg_launch(n, grid, sizeof(float2) * ((size_t)n + (size_t)T * (n + E + 1)), st, A));
  } else {
    dim3 grid((A.ncols + A.T - 1) / A.T, 1, 1);
    CK(A.flen.n1 ? kw_axis_launch_1(grid, p->smem_axis_ops, st, A) : kw_axis_launch_0(grid, p->smem_axis_ops, st, A));
  }
  CK(cudaGetLastError());
  return ev_end(p, st, KW_K_AXIS_OPS, slot);
}

// Source-kappa pass over the scattered source fields of step t
// (kspace_solver.py:91-98): rows -> [y] -> x with source_kappa -> [y^-1].
static int enqueue_sources(kw_plan* p, int t, cudaStream_t st) {
  const bool three = p->D == 3;
  int bufs[4], nb = 0;
  if (p->srcp_on) bufs[nb++] = B_SRCP;
  for (int a = 0; a < p->D; ++a)
    if (p->srcu_on[a]) bufs[nb++] = B_SRCU0 + a;
  if (!nb) return KW_OK;
  int rc;
  if ((rc = launch_rows(p, ST_SRC, 0, t, 0, st))) return rc;
  if (three && (rc = launch_axis_plain(p, 1, 0, bufs, nb, st))) return rc;
  AxisJob jobs[KW_MAX_JOBS];
  for (int i = 0; i < nb; ++i) jobs[i] = AxisJob{bufs[i], bufs[i], OP_SKAPPA, 0};
  if ((rc = launch_axis_ops(p, jobs, nb, st))) return rc;
  if (three && (rc = launch_axis_plain(p, 1, 1, bufs, nb, st))) return rc;
  return KW_OK;
}

static void set_step_flags(kw_plan* p, int t) {
  const HostSrc& hp = p->hsrc[KW_S_P0];
  p->srcp_on = hp.set && hp.mode == KW_SRC_ADDITIVE && t < hp.len;
  for (int a = 0; a < 3; ++a) {
    const HostSrc& h = p->hsrc[KW_S_U0 + a];
    p->srcu_on[a] = a < p->D && h.set && h.mode == KW_SRC_ADDITIVE && t < h.len;
  }
  // bit a: u_a on the pressure grid is recorded (its spectrum buffer exists)
  p->rec_us = (t >= p->g.record_start) ? (p->record_mask >> KW_R_UX) & 0x7 : 0;
  p->init_r2c = 0;
}

static int enqueue_step(kw_plan* p, int t, bool last, cudaStream_t st) {
  const int D = p->D;
  const bool three = D == 3;
  int rc;
  const int SB[3] = {0, 1, 2};
  const int PB[1] = {B_P};
  // work spectra plus the recorded unstaggered-velocity spectra
  int SUB[6], nus = 0;
  for (int a = 0; a < D; ++a) SUB[a] = a;
  for (int a = 0; a < D; ++a)
    if ((p->record_mask >> (KW_R_UX + a)) & 1) SUB[D + nus++] = B_US0 + a;
  AxisJob jobs[KW_MAX_JOBS];
  const bool has_p0 = !p->hfield[KW_F_P0].empty();
  set_step_flags(p, t);
  if (t == 0 && has_p0) {
    // initial condition override (kspace_solver.py:725-733); sources of step 0 are overwritten
    const int rec_us = p->rec_us;
    p->srcp_on = 0;
    p->srcu_on[0] = p->srcu_on[1] = p->srcu_on[2] = 0;
    p->rec_us = 0;
    if (p->smooth && !p->p0s_ready) {
      // p0 smoothing with restore_max (kwave/utils/filters.py:549-615), once per plan
      const long long n = p->ntot;
      const int grid = (int)std::min<long long>((n + 255) / 256, 4 * (long long)p->nsm);
      CK(cudaMemsetAsync(p->d_maxes, 0, 2 * sizeof(unsigned int), st));
      k_absmax<<<grid, 256, 0, st>>>(p->d_field[KW_F_P0], n, p->d_maxes);
      CK(cudaGetLastError());
      CK(cudaMemcpyAsync(p->d_p0s, p->d_field[KW_F_P0], n * sizeof(float), cudaMemcpyDeviceToDevice, st));
      if ((rc = launch_rows(p, ST_P0FFT, 0, t, 0, st))) return rc;
      if (three && (rc = launch_axis_plain(p, 1, 0, PB, 1, st))) return rc;
      jobs[0] = AxisJob{B_P, B_P, OP_WIN, 0};
      if ((rc = launch_axis_ops(p, jobs, 1, st))) return rc;
      if (three && (rc = launch_axis_plain(p, 1, 1, PB, 1, st))) return rc;
      if ((rc = launch_rows(p, ST_P0BACK, 0, t, 0, st))) return rc;
      k_absmax<<<grid, 256, 0, st>>>(p->d_p0s, n, p->d_maxes + 1);
      CK(cudaGetLastError());
      k_ratio<<<1, 32, 0, st>>>(p->d_maxes, p->d_maxes + 1, p->d_p0scale);
      CK(cudaGetLastError());
      p->p0s_ready = true;
    }
    if ((rc = launch_rows(p, ST_INIT, 0, t, 1, st))) return rc;
    if (three && (rc = launch_axis_plain(p, 1, 0, PB, 1, st))) return rc;
    for (int a = 0; a < D; ++a) jobs[a] = AxisJob{B_P, a, OP_GRAD, a};
    if ((rc = launch_axis_ops(p, jobs, D, st))) return rc;
    if (three && (rc = launch_axis_plain(p, 1, 1, SB, D, st))) return rc;
    p->init_r2c = rec_us;
    if ((rc = launch_rows(p, ST_U, 1, t, 0, st))) return rc;
    p->init_r2c = 0;
    if (rec_us) {
      // velocity on the pressure grid at t = 0 (kspace_solver.py:740-743)
      if (three && (rc = launch_axis_plain(p, 1, 0, SB, D, st))) return rc;
      int nj = 0;
      for (int a = 0; a < D; ++a)
        if ((rec_us >> a) & 1) jobs[nj++] = AxisJob{a, B_US0 + a, OP_UNSTAG, a};
      if ((rc = launch_axis_ops(p, jobs, nj, st))) return rc;
      if (three && (rc = launch_axis_plain(p, 1, 1, SUB + D, nus, st))) return rc;
      p->rec_us = rec_us;
      if ((rc = launch_rows(p, ST_UREC, 0, t, 0, st))) return rc;
      p->rec_us = 0;
    }
    return KW_OK;
  }
  if ((rc = enqueue_sources(p, t, st))) return rc;
  // momentum
  for (int a = 0; a < D; ++a) jobs[a] = AxisJob{B_P, a, OP_GRAD, a};
  if ((rc = launch_axis_ops(p, jobs, D, st))) return rc;
  if (three && (rc = launch_axis_plain(p, 1, 1, SB, D, st))) return rc;
  if ((rc = launch_rows(p, ST_U, 0, t, 0, st))) return rc;
  // mass conservation (+ velocity on the pressure grid when recorded)
  if (three && (rc = launch_axis_plain(p, 1, 0, SB, D, st))) return rc;
  int nj = 0;
  for (int a = 0; a < D; ++a) {
    jobs[nj++] = AxisJob{a, a, OP_DIV, a};
    if ((p->rec_us >> a) & 1) jobs[nj++] = AxisJob{a, B_US0 + a, OP_UNSTAG, a};
  }
  if ((rc = launch_axis_ops(p, jobs, nj, st))) return rc;
  if (three && (rc = launch_axis_plain(p, 1, 1, SUB, p->rec_us ? D + nus : D, st))) return rc;
  const bool powerlaw = p->g.absorb_mode == 1;
  if ((rc = launch_rows(p, ST_RHO, 0, t, (!powerlaw && last) ? 1 : 0, st))) return rc;
  if (powerlaw) {
    const int nb = p->g.dispersion ? 2 : 1;
    if (three && (rc = launch_axis_plain(p, 1, 0, SB, nb, st))) return rc;
    jobs[0] = AxisJob{0, 0, OP_NAB1, 0};
    jobs[1] = AxisJob{1, 1, OP_NAB2, 0};
    if ((rc = launch_axis_ops(p, jobs, nb, st))) return rc;
    if (three && (rc = launch_axis_plain(p, 1, 1, SB, nb, st))) return rc;
    if ((rc = launch_rows(p, ST_EOS, 0, t, last ? 1 : 0, st))) return rc;
  }
  if (three && (rc = launch_axis_plain(p, 1, 0, PB, 1, st))) return rc;
  return KW_OK;
}

// ---------------------------------------------------------------------------
// step graphs
// ---------------------------------------------------------------------------
// Launch sequence of step t as a key: two steps with the same key launch the
// same kernels with the same arguments apart from the step index, which the
// row stages of a captured step read from the device counter.
static int step_key(kw_plan* p, int t) {
  set_step_flags(p, t);
  return p->srcp_on | (p->srcu_on[0] << 1) | (p->srcu_on[1] << 2) | (p->srcu_on[2] << 3) | (p->rec_us << 4) |
         ((t >= p->g.record_start ? 1 : 0) << 7);
}

// Steps that run as plain launches: the last step of a run (it writes p to
// real space), the t = 0 initial-condition override, and every step while
// per-launch timing is on.
static bool step_eager(const kw_plan* p, int t, int end) {
  return !p->use_graphs || p->timing || t == end - 1 || (t == 0 && !p->hfield[KW_F_P0].empty());
}

static void drop_graphs(kw_plan* p) {
  for (auto& g : p->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  p->graphs.clear();
}

// Captured step graph for the key of step t (captured on first use).
static int step_graph(kw_plan* p, int t, kw_plan::StepGraph** out) {
  const int key = step_key(p, t);
  for (auto& g : p->graphs)
    if (g.key == key) {
      *out = &g;
      return KW_OK;
    }
  if (!p->cap_stream) CK(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
  const long long l0 = p->launches;
  CK(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeRelaxed));
  p->capturing = true;
  int rc = enqueue_step(p, t, false, p->cap_stream);
  p->capturing = false;
  if (!rc) {
    k_step_tick<<<1, 1, 0, p->cap_stream>>>(p->d_tstep);
    if (cudaGetLastError() != cudaSuccess) rc = fail(KW_ERR_CUDA, "step counter launch failed during capture");
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(p->cap_stream, &graph);
  const long long nl = p->launches - l0 + 1;
  p->launches = l0;
  if (!rc && ec != cudaSuccess) rc = fail(KW_ERR_CUDA, "step capture: %s", cudaGetErrorString(ec));
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(KW_ERR_CUDA, "step graph instantiation: %s", cudaGetErrorString(ei));
  }
  p->graphs.push_back(kw_plan::StepGraph{key, graph, exec, nl});
  *out = &p->graphs.back();
  return KW_OK;
}

// Point the device counter at step t (if the stream will not already hold t there).
static int step_counter_to(kw_plan* p, int t, cudaStream_t st) {
  if (p->tstep_val == t) return KW_OK;
  k_step_set<<<1, 1, 0, st>>>(p->d_tstep, t);
  CK(cudaGetLastError());
  p->launches++;
  p->tstep_val = t;
  return KW_OK;
}

static int run_step(kw_plan* p, int t, int end, cudaStream_t st) {
  if (step_eager(p, t, end)) return enqueue_step(p, t, t == end - 1, st);
  kw_plan::StepGraph* g = nullptr;
  int rc = step_graph(p, t, &g);
  if (!rc) rc = step_counter_to(p, t, st);
  if (rc) return rc;
  CK(cudaGraphLaunch(g->exec, st));
  p->tstep_val = t + 1;
  p->launches += g->nlaunch;
  return KW_OK;
}

// plain_last == false (autotuning only): the last step is a graph step too and
// leaves p in spectral form only.
static size_t ckpt_floats(const kw_plan* p) { return 2 * (size_t)p->D * p->ntot + 2 * (size_t)p->spec_elems; }

// Copy the state carried into step t + 1 (u_i, rho_i, spectrum of p) to or
// from checkpoint slot s.
static int ckpt_copy(kw_plan* p, int s, bool save, cudaStream_t st) {
  float* base = p->ckpt[s];
  const size_t nf = (size_t)p->ntot * sizeof(float);
  for (int a = 0; a < p->D; ++a) {
    float* cu = base + (size_t)a * p->ntot;
    float* cr = base + (size_t)(p->D + a) * p->ntot;
    CK(cudaMemcpyAsync(save ? cu : p->d_u[a], save ? p->d_u[a] : cu, nf, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(save ? cr : p->d_rho[a], save ? p->d_rho[a] : cr, nf, cudaMemcpyDeviceToDevice, st));
  }
  float* cs = base + 2 * (size_t)p->D * p->ntot;
  CK(cudaMemcpyAsync(save ? (void*)cs : (void*)p->d_S[B_P], save ? (void*)p->d_S[B_P] : (void*)cs,
                     (size_t)p->spec_elems * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  return KW_OK;
}

static int plan_run(kw_plan* p, int nsteps, cudaStream_t st, bool plain_last) {
  const int end = std::min(p->g.Nt, p->t + nsteps);
  const int eend = plain_last ? end : end + 1;
  for (int t = p->t; t < end; ++t) {
    int rc = run_step(p, t, eend, st);
    if (rc) return rc;
    p->t = t + 1;
    if (p->ckpt_K > 0 && t % p->ckpt_K == 0) {
      const int s = t / p->ckpt_K;
      if ((rc = ckpt_copy(p, s, true, st))) return rc;
      p->ckpt_ok[s] = 1;
    }
  }
  return KW_OK;
}

int32_t kw_plan_run(kw_plan* p, int32_t nsteps, void* stream) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_run before kw_plan_finalize");
  if (nsteps < 0) return fail(KW_ERR_INVALID, "nsteps < 0");
  return plan_run(p, nsteps, reinterpret_cast<cudaStream_t>(stream), true);
}

// Times the plan's first `nsteps` steps for each candidate geometry of the
// run-time-length kernels (tile columns T in {2, 4, 8, 16}, rows per block
// R in {R0/2, R0, 2 R0}), keeps the fastest and rewinds the plan to t = 0.
// Results do not depend on the choice.
int32_t kw_plan_autotune(kw_plan* p, int32_t nsteps, void* stream, int32_t* T_out, int32_t* R_out) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_autotune before kw_plan_finalize");
  if (p->t != 0) return fail(KW_ERR_STATE, "kw_plan_autotune needs a plan at t = 0 (kw_plan_reset first)");
  bool gen_axis = false;
  for (int a = 0; a < p->D - 1; ++a) gen_axis |= !p->tma_axis[a] && !p->axis_reg[a];
  const bool gen_rows = !p->rows_reg;
  const int k = std::min(std::max(2, (int)nsteps), p->g.Nt - 1);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if ((gen_axis || gen_rows) && k >= 2) {
    const int R0 = default_rows_per_block(p);
    std::vector<int> Ts = gen_axis ? std::vector<int>{2, 4, 8, 16} : std::vector<int>{0};
    std::vector<int> Rs{R0};
    if (gen_rows) {
      if (R0 > 1) Rs.push_back(std::max(1, R0 / 2));
      if (rows_smem_bytes(p, 2 * R0) <= 200 * 1024) Rs.push_back(2 * R0);
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int bestT = 0, bestR = R0, rc = KW_OK;
    const bool timing = p->timing;
    p->timing = false;
    for (int T : Ts) {
      for (int R : Rs) {
        set_generic_geometry(p, T, R);
        drop_graphs(p);
        // one untimed pass captures the step graphs; the timed steps follow
        // the t = 0 step and are all graph steps
        if ((rc = plan_run(p, 1 + k, st, false)) || (rc = kw_plan_reset(p)) || (rc = plan_run(p, 1, st, false)))
          break;
        float ms = 0.f;
        if (cudaEventRecord(e0, st) != cudaSuccess) rc = fail(KW_ERR_CUDA, "autotune event");
        if (!rc) rc = plan_run(p, k, st, false);
        if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
          rc = fail(KW_ERR_CUDA, "autotune timing");
        if (!rc) rc = kw_plan_reset(p);
        if (rc) break;
        if (ms < best) {
          best = ms;
          bestT = T;
          bestR = R;
        }
      }
      if (rc) break;
    }
    p->timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_generic_geometry(p, bestT, bestR);
    drop_graphs(p);
    if (rc) return rc;
    if ((rc = kw_plan_reset(p))) return rc;
  }
  if (T_out) *T_out = p->D > 1 ? p->T_axis[0] : 0;
  if (R_out) *R_out = p->R;
  return KW_OK;
}

static int check_device_error();

int32_t kw_plan_set_checkpoints(kw_plan* p, int32_t interval) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_set_checkpoints before kw_plan_finalize");
  if (interval < 0) return fail(KW_ERR_INVALID, "checkpoint interval < 0");
  if (p->t != 0) return fail(KW_ERR_STATE, "kw_plan_set_checkpoints needs the plan at t = 0");
  CK(cudaDeviceSynchronize());
  for (float* c : p->ckpt) dfree_last(p, c);
  p->ckpt.clear();
  p->ckpt_ok.clear();
  p->ckpt_K = 0;
  if (interval == 0) return KW_OK;
  const int nslot = (p->g.Nt - 1) / interval + 1;
  p->ckpt.assign(nslot, nullptr);
  for (int s = 0; s < nslot; ++s) {
    int rc = dalloc(p, &p->ckpt[s], ckpt_floats(p));
    if (rc) {
      p->ckpt.resize(s);
      for (float* c : p->ckpt) dfree_last(p, c);
      p->ckpt.clear();
      return rc;
    }
  }
  p->ckpt_ok.assign(nslot, 0);
  p->ckpt_K = interval;
  return KW_OK;
}

namespace {
// Adjoint state and work buffers of one kw_plan_adjoint call (freed on return).
struct AdjBufs {
  std::vector<void*> mem;
  ~AdjBufs() {
    for (void* m : mem) cudaFree(m);
  }
  int get(float** out, size_t count) {
    void* ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, count * sizeof(float));
    if (e != cudaSuccess)
      return fail(e == cudaErrorMemoryAllocation ? KW_ERR_OOM : KW_ERR_CUDA, "cudaMalloc(%zu): %s",
                  count * sizeof(float), cudaGetErrorString(e));
    mem.push_back(ptr);
    *out = static_cast<float*>(ptr);
    return KW_OK;
  }
};
}  // namespace

// Exchanges the plan's state and p series with the adjoint's buffers, so that
// the row stages (which read the plan) see the adjoint state.
static void adj_swap(kw_plan* p, float*& lp, float** lu, float** lr, float*& res) {
  std::swap(p->d_p, lp);
  for (int a = 0; a < p->D; ++a) {
    std::swap(p->d_u[a], lu[a]);
    std::swap(p->d_rho[a], lr[a]);
  }
  std::swap(p->d_rec[KW_R_P], res);
}

// The gradient of <residual, recorded p> for the lossless, source-free loop:
// the transposed steps t = Nt-1 .. 1 and the transposed t = 0 override
// (adjoint_body in kw_kernels.cu) on the run-time-length row kernels, with the
// adjoint state in buffers of its own.  With grad_c, the forward density sum
// of every step is regenerated from the checkpoints, segment by segment from
// the last (restore slot s, rerun its steps, keep sum_i rho_i of each), and
// the segment's adjoint steps accumulate the sound-speed gradient.
int32_t kw_plan_adjoint(kw_plan* p, const float* residual, int64_t n, float* grad_p0, float* grad_c, void* stream) {
  if (!p || !residual || !grad_p0) return fail(KW_ERR_INVALID, "kw_plan_adjoint: null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_adjoint before kw_plan_finalize");
  if (p->g.absorb_mode != 0 || p->g.nonlinear)
    return fail(KW_ERR_UNSUPPORTED, "the adjoint covers the lossless loop (no absorption, no B/A)");
  for (int s = 0; s < 6; ++s)
    if (p->hsrc[s].set) return fail(KW_ERR_UNSUPPORTED, "the adjoint covers the source-free loop");
  if (!(p->record_mask & (1 << KW_R_P)) || p->nslots == 0)
    return fail(KW_ERR_UNSUPPORTED, "the adjoint needs a sensor recording p");
  if (n != (int64_t)p->nrec * p->nslots)
    return fail(KW_ERR_INVALID, "residual has %lld values, expected %lld", (long long)n, (long long)p->nrec * p->nslots);
  const int K = p->ckpt_K;
  if (grad_c) {
    if (p->smooth) return fail(KW_ERR_UNSUPPORTED, "the sound-speed gradient needs p0 smoothing off");
    if (p->hfield[KW_F_P0].empty()) return fail(KW_ERR_STATE, "the sound-speed gradient needs the forward's p0");
    if (K <= 0) return fail(KW_ERR_STATE, "the sound-speed gradient needs checkpoints (kw_plan_set_checkpoints)");
    if (p->t != p->g.Nt) return fail(KW_ERR_STATE, "the sound-speed gradient needs the forward run to t = Nt");
    for (char ok : p->ckpt_ok)
      if (!ok) return fail(KW_ERR_STATE, "a checkpoint of the forward run is missing (run from t = 0 after setting them)");
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int D = p->D;
  const bool three = D == 3;
  const size_t nt = (size_t)p->ntot;
  AdjBufs B;
  float *lp, *lu[3] = {nullptr, nullptr, nullptr}, *lr[3] = {nullptr, nullptr, nullptr}, *res, *gacc = nullptr;
  float* seg = nullptr;
  int rc = B.get(&lp, nt);
  for (int a = 0; a < D && !rc; ++a)
    if (!(rc = B.get(&lu[a], nt))) rc = B.get(&lr[a], nt);
  if (!rc) rc = B.get(&res, (size_t)n);
  if (!rc && grad_c && !(rc = B.get(&gacc, nt))) rc = B.get(&seg, (size_t)K * nt);
  if (rc) return rc;
  CK(cudaMemsetAsync(lp, 0, nt * sizeof(float), st));
  for (int a = 0; a < D; ++a) {
    CK(cudaMemsetAsync(lu[a], 0, nt * sizeof(float), st));
    CK(cudaMemsetAsync(lr[a], 0, nt * sizeof(float), st));
  }
  if (gacc) CK(cudaMemsetAsync(gacc, 0, nt * sizeof(float), st));
  {
    // sensor-major (n_points, n_rec) -> the time-major series layout
    std::vector<float> tm((size_t)n);
    for (int s = 0; s < p->nslots; ++s)
      for (int t = 0; t < p->nrec; ++t) tm[(size_t)t * p->nslots + s] = residual[(size_t)s * p->nrec + t];
    CK(cudaMemcpyAsync(res, tm.data(), tm.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  const bool timing = p->timing;
  p->timing = false;
  const int SB[3] = {0, 1, 2};
  AxisJob gj[3], dj[3];
  for (int a = 0; a < D; ++a) {
    gj[a] = AxisJob{a, a, OP_GRAD, a};
    dj[a] = AxisJob{a, a, OP_DIV, a};
  }
  const long long grid = std::min<long long>(((long long)nt + 255) / 256, 8LL * p->nsm);
  auto dsum = [&](float* out) -> int {
    k_density_sum<<<(int)grid, 256, 0, st>>>(out, p->d_rho[0], p->d_rho[1], D == 3 ? p->d_rho[2] : nullptr,
                                             (long long)nt);
    CK(cudaGetLastError());
    p->launches++;
    return KW_OK;
  };
  // adjoint steps t = hi .. lo (descending), the plan's buffers swapped for the adjoint's
  auto adj_steps = [&](int hi, int lo, int t_base) -> int {
    adj_swap(p, lp, lu, lr, res);
    int r = KW_OK;
    for (int t = hi; t >= lo && !r; --t) {
      p->adj_fsum = seg ? seg + (size_t)(t - t_base) * nt : nullptr;
      p->adj_gacc = gacc;
      if ((r = launch_rows(p, ST_ADJ_A, 0, t, 0, st))) break;
      p->adj_fsum = nullptr;
      p->adj_gacc = nullptr;
      if (three && (r = launch_axis_plain(p, 1, 0, SB, D, st))) break;
      if ((r = launch_axis_ops(p, gj, D, st))) break;
      if (three && (r = launch_axis_plain(p, 1, 1, SB, D, st))) break;
      if ((r = launch_rows(p, ST_ADJ_B, 0, t, 0, st))) break;
      if (three && (r = launch_axis_plain(p, 1, 0, SB, D, st))) break;
      if ((r = launch_axis_ops(p, dj, D, st))) break;
      if (three && (r = launch_axis_plain(p, 1, 1, SB, D, st))) break;
      r = launch_rows(p, ST_ADJ_C, 0, t, 0, st);
    }
    p->adj_fsum = nullptr;
    p->adj_gacc = nullptr;
    adj_swap(p, lp, lu, lr, res);
    return r;
  };
  const int Nt = p->g.Nt;
  if (!grad_c) {
    rc = adj_steps(Nt - 1, 1, 0);
  } else {
    // forward recomputation runs as plain launches and records nothing
    float* rec_p = p->d_rec[KW_R_P];
    p->d_rec[KW_R_P] = nullptr;
    const int nseg = (Nt - 1) / K + 1;
    for (int s = nseg - 1; s >= 0 && !rc; --s) {
      const int t0 = s * K, t1 = std::min(t0 + K - 1, Nt - 1);
      if ((rc = ckpt_copy(p, s, false, st))) break;
      if ((rc = dsum(seg))) break;
      for (int t = t0 + 1; t <= t1 && !rc; ++t)
        if (!(rc = enqueue_step(p, t, t == Nt - 1, st))) rc = dsum(seg + (size_t)(t - t0) * nt);
      if (!rc) rc = adj_steps(t1, std::max(t0, 1), t0);
    }
    p->d_rec[KW_R_P] = rec_p;
  }
  if (!rc) {
    adj_swap(p, lp, lu, lr, res);
    rc = launch_rows(p, ST_ADJ_D, 0, 0, 0, st);
    if (!rc && three) rc = launch_axis_plain(p, 1, 0, SB, D, st);
    if (!rc) rc = launch_axis_ops(p, dj, D, st);
    if (!rc && three) rc = launch_axis_plain(p, 1, 1, SB, D, st);
    p->adj_gacc = gacc;
    if (!rc) rc = launch_rows(p, ST_ADJ_E, 0, 0, 0, st);
    p->adj_gacc = nullptr;
    adj_swap(p, lp, lu, lr, res);
  }
  p->timing = timing;
  if (rc) return rc;
  CK(cudaStreamSynchronize(st));
  if ((rc = check_device_error())) return rc;
  CK(cudaMemcpy(grad_p0, lp, nt * sizeof(float), cudaMemcpyDeviceToHost));
  if (grad_c) CK(cudaMemcpy(grad_c, gacc, nt * sizeof(float), cudaMemcpyDeviceToHost));
  return kw_plan_reset(p);
}

int32_t kw_plan_adjoint_p0(kw_plan* p, const float* residual, int64_t n, float* grad, void* stream) {
  return kw_plan_adjoint(p, residual, n, grad, nullptr, stream);
}

int32_t kw_plan_set_wait_test(kw_plan* p, int32_t enable) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (!p->finalized) return fail(KW_ERR_STATE, "kw_plan_set_wait_test before kw_plan_finalize");
  if (enable && !p->rows_tma)
    return fail(KW_ERR_UNSUPPORTED, "the wait test needs the bulk-fed row stages (a power-of-two last axis)");
  CK(cudaDeviceSynchronize());
  p->wait_test = enable != 0;
  drop_graphs(p);  // captured steps hold the launch parameters
  return KW_OK;
}

int32_t kw_plan_set_graphs(kw_plan* p, int32_t enable) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  p->use_graphs = enable != 0;
  return KW_OK;
}

// ---------------------------------------------------------------------------
// batches: several plans advanced together, one graph launch per step
// ---------------------------------------------------------------------------
struct kw_batch {
  std::vector<kw_plan*> plans;
  struct Graph {
    std::vector<int> keys;     // per plan: step key, or -1 when the plan does not step
    std::vector<char> grouped; // per plan: its passes run inside the grouped launches
    std::vector<long long> nl; // per ungrouped plan: launches of its step graph
    cudaGraph_t graph;         // the step graph (kept as the body of loop graphs)
    cudaGraphExec_t exec;
    cudaGraphExec_t loop_exec; // the step graph in a device-side while loop, or null
    long long nlaunch;         // grouped launches per replay
  };
  std::vector<Graph> graphs;
  std::vector<void*> allocs;
  cudaStream_t cap = nullptr;
  long long launches = 0;
  // steps whose key vector has no batch graph yet and differs from the
  // previous step's: the members' own step graphs on side streams
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_done;
  cudaEvent_t fork_ev = nullptr;
  std::vector<int> last_keys;
  int repeat = 0;
  // runs of steps with one key vector: one launch of a graph that loops over
  // the step graph on the device (KWAVE_GB300_BATCH_LOOPS=0 or
  // kw_batch_set_loops(b, 0): one launch per step)
  bool loops = true;
  int* d_loop = nullptr;      // passes left in the running loop graph
  long long graph_launches = 0;
};

int32_t kw_batch_create(kw_plan* const* plans, int32_t n, kw_batch** out) {
  if (!out || n < 1 || !plans) return fail(KW_ERR_INVALID, "kw_batch_create: need at least one plan");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!plans[i]) return fail(KW_ERR_INVALID, "kw_batch_create: plan %d is null", i);
    if (!plans[i]->finalized) return fail(KW_ERR_STATE, "kw_batch_create: plan %d is not finalized", i);
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return fail(KW_ERR_INVALID, "kw_batch_create: plan %d given twice", i);
  }
  kw_batch* b = new kw_batch;
  b->plans.assign(plans, plans + n);
  {
    const char* env = getenv("KWAVE_GB300_BATCH_LOOPS");
    b->loops = !(env && env[0] == '0');
  }
  // step graphs of batch members become child graphs: capture them with plain
  // stream-order edges between their kernels
  for (kw_plan* p : b->plans)
    if (p->pdl) {
      p->pdl = false;
      drop_graphs(p);
    }
  *out = b;
  return KW_OK;
}

static int batch_upload(kw_batch* b, const void* host, size_t bytes, void** out) {
  void* d = nullptr;
  CK(cudaMalloc(&d, bytes));
  b->allocs.push_back(d);
  CK(cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice));
  *out = d;
  return KW_OK;
}

// The graph of one batch step for the given per-plan keys (built on first use).
// The steps of plans whose passes are all generic are recorded, and launch k
// of every such plan runs in one grouped launch (rows and axis passes apart);
// the other plans join as child graphs of their own step graphs.
static int batch_graph(kw_batch* b, const std::vector<int>& keys, kw_batch::Graph** out) {
  for (auto& g : b->graphs)
    if (g.keys == keys) {
      *out = &g;
      return KW_OK;
    }
  const size_t n = keys.size();
  std::vector<std::vector<kw_plan::LaunchRec>> lists(n);
  kw_batch::Graph G;
  G.keys = keys;
  G.grouped.assign(n, 0);
  G.nl.assign(n, 0);
  G.graph = nullptr;
  G.exec = nullptr;
  G.loop_exec = nullptr;
  G.nlaunch = 0;
  int rc;
  for (size_t i = 0; i < n; ++i) {
    if (keys[i] < 0) continue;
    kw_plan* p = b->plans[i];
    p->rec_list = &lists[i];
    p->capturing = true;
    rc = enqueue_step(p, p->t, false, nullptr);
    p->rec_list = nullptr;
    p->capturing = false;
    if (rc) return rc;
    // only plans created for grouping (KW_DESC_GENERIC_FFT): on the same
    // kernels, separate branches measured faster than grouped launches
    bool ok = !lists[i].empty() && (p->g.flags & KW_DESC_GENERIC_FFT);
    for (auto& r : lists[i]) ok = ok && r.kind != 2;
    G.grouped[i] = ok;
  }
  struct Pending {
    int kind, m, total;
    size_t smem;
    void* params;
    int4* blk;
    int sched;  // FFT schedule family of the grouped kernel (kw_generic.cuh)
  };
  std::vector<Pending> pend;
  std::vector<int*> ticks;
  size_t maxlen = 0;
  for (size_t i = 0; i < n; ++i)
    if (G.grouped[i]) {
      maxlen = std::max(maxlen, lists[i].size());
      ticks.push_back(b->plans[i]->d_tstep);
    }
  // launch j of the members: one grouped launch per kind (rows, axis) and FFT
  // schedule family
  for (size_t j = 0; j < maxlen; ++j)
    for (int ks = 0; ks < 4; ++ks) {
      const int kind = ks >> 1, sched = ks & 1;
      std::vector<RowsParams> rp;
      std::vector<AxisParams> ap;
      std::vector<int4> blk;
      long long total = 0;
      size_t smem = 0;
      for (size_t i = 0; i < n; ++i) {
        if (!G.grouped[i] || lists[i].size() <= j || lists[i][j].kind != kind) continue;
        const kw_plan::LaunchRec& r = lists[i][j];
        if ((kind == 0 ? r.rp.flen.n1 : r.ap.flen.n1) != 0 ? !sched : sched) continue;
        blk.push_back(make_int4((int)total, r.gx, r.gy, 0));
        if (kind == 0)
          rp.push_back(r.rp);
        else
          ap.push_back(r.ap);
        total += (long long)r.gx * r.gy * r.gz;
        smem = std::max(smem, r.smem);
      }
      if (blk.empty()) continue;
      if (total >= (1LL << 31)) return fail(KW_ERR_UNSUPPORTED, "grouped launch of %lld blocks", total);
      const int m = (int)blk.size();
      blk.push_back(make_int4((int)total, 0, 0, 0));
      Pending q{kind, m, (int)total, smem, nullptr, nullptr, sched};
      if (kind == 0)
        rc = batch_upload(b, rp.data(), rp.size() * sizeof(RowsParams), &q.params);
      else
        rc = batch_upload(b, ap.data(), ap.size() * sizeof(AxisParams), &q.params);
      void* dblk = nullptr;
      if (!rc) rc = batch_upload(b, blk.data(), blk.size() * sizeof(int4), &dblk);
      if (rc) return rc;
      q.blk = static_cast<int4*>(dblk);
      pend.push_back(q);
    }
  int** dticks = nullptr;
  if (!ticks.empty()) {
    void* d = nullptr;
    if ((rc = batch_upload(b, ticks.data(), ticks.size() * sizeof(int*), &d))) return rc;
    dticks = static_cast<int**>(d);
  }
  // ungrouped plans: their own step graphs
  std::vector<kw_plan::StepGraph*> sg(n, nullptr);
  for (size_t i = 0; i < n; ++i)
    if (keys[i] >= 0 && !G.grouped[i]) {
      if ((rc = step_graph(b->plans[i], b->plans[i]->t, &sg[i]))) return rc;
      G.nl[i] = sg[i]->nlaunch;
    }
  if (!b->cap) CK(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
  CK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
  cudaError_t elaunch = cudaSuccess;
  for (const Pending& q : pend) {
    const RowsParams* rq = static_cast<const RowsParams*>(q.params);
    const AxisParams* aq = static_cast<const AxisParams*>(q.params);
    cudaError_t e;
    if (q.kind == 0)
      e = q.sched ? kw_rows_group_launch_1(q.total, q.smem, b->cap, rq, q.blk, q.m)
                  : kw_rows_group_launch_0(q.total, q.smem, b->cap, rq, q.blk, q.m);
    else
      e = q.sched ? kw_axis_group_launch_1(q.total, q.smem, b->cap, aq, q.blk, q.m)
                  : kw_axis_group_launch_0(q.total, q.smem, b->cap, aq, q.blk, q.m);
    if (elaunch == cudaSuccess) elaunch = e;
  }
  if (dticks) k_step_tick_group<<<((int)ticks.size() + 127) / 128, 128, 0, b->cap>>>(dticks, (int)ticks.size());
  const cudaError_t el = elaunch != cudaSuccess ? elaunch : cudaGetLastError();
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(b->cap, &graph);
  if (el != cudaSuccess || ec != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(KW_ERR_CUDA, "batch capture: %s", cudaGetErrorString(el != cudaSuccess ? el : ec));
  }
  G.nlaunch = (long long)pend.size() + (dticks ? 1 : 0);
  for (size_t i = 0; i < n; ++i) {
    if (!sg[i]) continue;
    cudaGraphNode_t node;
    const cudaError_t e = cudaGraphAddChildGraphNode(&node, graph, nullptr, 0, sg[i]->graph);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      return fail(KW_ERR_CUDA, "batch graph: %s", cudaGetErrorString(e));
    }
  }
  const cudaError_t ei = cudaGraphInstantiate(&G.exec, graph, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(KW_ERR_CUDA, "batch graph instantiation: %s", cudaGetErrorString(ei));
  }
  G.graph = graph;
  b->graphs.push_back(G);
  *out = &b->graphs.back();
  return KW_OK;
}

// The loop graph of a batch step graph: a conditional while node whose body
// is the step graph followed by k_loop_tick, so that one launch runs as many
// steps as k_loop_set put in d_loop.
static int batch_loop_graph(kw_batch* b, kw_batch::Graph* g) {
  if (g->loop_exec) return KW_OK;
  if (!b->d_loop) CK(cudaMalloc(&b->d_loop, sizeof(int)));
  cudaGraph_t lg = nullptr;
  CK(cudaGraphCreate(&lg, 0));
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t cn, child, tick;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, lg, 1, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&cn, lg, nullptr, nullptr, 0, &cp);
  }
  if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&child, cp.conditional.phGraph_out[0], nullptr, 0, g->graph);
  if (e == cudaSuccess) {
    cudaKernelNodeParams kp = {};
    int* left = b->d_loop;
    void* args[2] = {&h, &left};
    kp.func = reinterpret_cast<void*>(k_loop_tick);
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = args;
    e = cudaGraphAddKernelNode(&tick, cp.conditional.phGraph_out[0], &child, 1, &kp);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->loop_exec, lg, 0);
  cudaGraphDestroy(lg);
  if (e != cudaSuccess) {
    g->loop_exec = nullptr;
    return fail(KW_ERR_CUDA, "batch loop graph: %s", cudaGetErrorString(e));
  }
  return KW_OK;
}

static kw_batch::Graph* find_batch_graph(kw_batch* b, const std::vector<int>& keys) {
  for (auto& g : b->graphs)
    if (g.keys == keys) return &g;
  return nullptr;
}

// One step of every stepping member through its own step graph, members
// spread over up to 16 side streams forked from and joined back into `st`.
static int batch_step_streams(kw_batch* b, const std::vector<int>& keys, cudaStream_t st) {
  const size_t n = b->plans.size();
  if (b->side.empty()) {
    const size_t ns = std::min<size_t>(n, 16);
    for (size_t s = 0; s < ns; ++s) {
      cudaStream_t x;
      cudaEvent_t e;
      CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
      b->side.push_back(x);
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      b->side_done.push_back(e);
    }
    CK(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
  }
  const size_t ns = b->side.size();
  std::vector<kw_plan::StepGraph*> sg(n, nullptr);
  int rc;
  for (size_t i = 0; i < n; ++i)
    if (keys[i] >= 0 && (rc = step_graph(b->plans[i], b->plans[i]->t, &sg[i]))) return rc;
  CK(cudaEventRecord(b->fork_ev, st));
  for (size_t s = 0; s < ns; ++s) CK(cudaStreamWaitEvent(b->side[s], b->fork_ev, 0));
  for (size_t i = 0; i < n; ++i) {
    if (keys[i] < 0) continue;
    kw_plan* p = b->plans[i];
    cudaStream_t x = b->side[i % ns];
    if ((rc = step_counter_to(p, p->t, x))) return rc;
    CK(cudaGraphLaunch(sg[i]->exec, x));
    p->tstep_val = p->t + 1;
    p->launches += sg[i]->nlaunch;
    p->t += 1;
  }
  for (size_t s = 0; s < ns; ++s) {
    CK(cudaEventRecord(b->side_done[s], b->side[s]));
    CK(cudaStreamWaitEvent(st, b->side_done[s], 0));
  }
  return KW_OK;
}

static int batch_run(kw_batch* b, int nsteps, cudaStream_t st, bool plain_last) {
  const size_t n = b->plans.size();
  std::vector<int> end(n), eend(n), keys(n);
  int span = 0;
  for (size_t i = 0; i < n; ++i) {
    kw_plan* p = b->plans[i];
    end[i] = std::min(p->g.Nt, p->t + nsteps);
    eend[i] = plain_last ? end[i] : end[i] + 1;
    span = std::max(span, end[i] - p->t);
  }
  for (int s = 0; s < span; ++s) {
    bool together = true;
    for (size_t i = 0; i < n; ++i) {
      kw_plan* p = b->plans[i];
      keys[i] = -1;
      if (p->t >= end[i]) continue;
      if (step_eager(p, p->t, eend[i])) {
        together = false;
        continue;
      }
      keys[i] = step_key(p, p->t);
    }
    int rc;
    if (!together) {
      // a step with plain launches somewhere: each plan on its own, in order
      for (size_t i = 0; i < n; ++i) {
        kw_plan* p = b->plans[i];
        if (p->t >= end[i]) continue;
        if ((rc = run_step(p, p->t, eend[i], st))) return rc;
        p->t += 1;
      }
      continue;
    }
    // a batch graph is built for a key vector seen on two steps in a row;
    // while members switch sources off one by one the keys change every
    // step, and those steps run on side streams instead of one-off graphs
    kw_batch::Graph* g = find_batch_graph(b, keys);
    if (!g) {
      if (keys == b->last_keys) {
        ++b->repeat;
      } else {
        b->last_keys = keys;
        b->repeat = 0;
      }
      if (b->repeat >= 1 && (rc = batch_graph(b, keys, &g))) return rc;
    }
    if (!g) {
      if ((rc = batch_step_streams(b, keys, st))) return rc;
      continue;
    }
    // how many steps from here keep this key vector (all of them graph steps)
    int m = 1;
    if (b->loops) {
      while (s + m < span) {
        bool same = true;
        for (size_t i = 0; i < n && same; ++i) {
          kw_plan* p = b->plans[i];
          const int t = p->t + m;
          if (keys[i] < 0) {
            same = t >= end[i];
          } else {
            same = t < end[i] && !step_eager(p, t, eend[i]) && step_key(p, t) == keys[i];
          }
        }
        if (!same) break;
        ++m;
      }
      if (m >= 4 && (rc = batch_loop_graph(b, g))) return rc;
    }
    for (size_t i = 0; i < n; ++i)
      if (keys[i] >= 0 && (rc = step_counter_to(b->plans[i], b->plans[i]->t, st))) return rc;
    if (m >= 4 && g->loop_exec) {
      k_loop_set<<<1, 1, 0, st>>>(b->d_loop, m);
      CK(cudaGetLastError());
      CK(cudaGraphLaunch(g->loop_exec, st));
      b->launches += 1 + (long long)m * (g->nlaunch + 1);
    } else {
      m = 1;
      CK(cudaGraphLaunch(g->exec, st));
      b->launches += g->nlaunch;
    }
    b->graph_launches += 1;
    for (size_t i = 0; i < n; ++i) {
      if (keys[i] < 0) continue;
      kw_plan* p = b->plans[i];
      p->tstep_val = p->t + m;
      p->launches += (long long)m * g->nl[i];
      p->t += m;
    }
    s += m - 1;
  }
  return KW_OK;
}

int32_t kw_batch_run(kw_batch* b, int32_t nsteps, void* stream) {
  if (!b) return fail(KW_ERR_INVALID, "null batch");
  if (nsteps < 0) return fail(KW_ERR_INVALID, "nsteps < 0");
  return batch_run(b, nsteps, reinterpret_cast<cudaStream_t>(stream), true);
}

static void batch_free_graphs(kw_batch* b) {
  for (auto& g : b->graphs) {
    if (g.loop_exec) cudaGraphExecDestroy(g.loop_exec);
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  b->graphs.clear();
}

static void batch_clear(kw_batch* b) {
  cudaDeviceSynchronize();
  batch_free_graphs(b);
  for (void* a : b->allocs) cudaFree(a);
  b->allocs.clear();
}

static int batch_reset(kw_batch* b) {
  for (kw_plan* p : b->plans) {
    int rc = kw_plan_reset(p);
    if (rc) return rc;
  }
  return KW_OK;
}

// Batch counterpart of kw_plan_autotune: one geometry for all members (tile
// columns T, rows per block R = f * R0 of each member), timed on the batch
// itself, since members running together favour other shapes than a member
// alone.
int32_t kw_batch_autotune(kw_batch* b, int32_t nsteps, void* stream, int32_t* T_out, int32_t* R_num,
                          int32_t* R_den) {
  if (!b) return fail(KW_ERR_INVALID, "null batch");
  for (kw_plan* p : b->plans)
    if (p->t != 0) return fail(KW_ERR_STATE, "kw_batch_autotune needs every plan at t = 0");
  bool any = false;
  for (kw_plan* p : b->plans) {
    bool g = !p->rows_reg;
    for (int a = 0; a < p->D - 1; ++a) g |= !p->tma_axis[a] && !p->axis_reg[a];
    any |= g;
  }
  int bestT = 0, bestN = 1, bestD = 1;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int rc = KW_OK;
  // timed steps: at most one less than the shortest member's Nt
  int k = std::max(2, (int)nsteps);
  for (kw_plan* p : b->plans) k = std::min(k, p->g.Nt - 1);
  if (any && k >= 2) {
    const int Ts[4] = {2, 4, 8, 16};
    const int fr[3][2] = {{1, 2}, {1, 1}, {2, 1}};  // R = R0 * num / den
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int ti = 0; ti < 4 && !rc; ++ti)
      for (int fi = 0; fi < 3 && !rc; ++fi) {
        bool fits = true;
        for (kw_plan* p : b->plans) {
          const int R = std::max(1, default_rows_per_block(p) * fr[fi][0] / fr[fi][1]);
          if (rows_smem_bytes(p, R) > 200 * 1024) fits = false;
        }
        if (!fits) continue;
        for (kw_plan* p : b->plans) {
          set_generic_geometry(p, Ts[ti], std::max(1, default_rows_per_block(p) * fr[fi][0] / fr[fi][1]));
          drop_graphs(p);
        }
        batch_clear(b);
        // one untimed pass builds the graphs; the timed steps follow the
        // t = 0 step and are all graph steps
        if ((rc = batch_run(b, 1 + k, st, false)) || (rc = batch_reset(b)) || (rc = batch_run(b, 1, st, false))) break;
        float ms = 0.f;
        if (cudaEventRecord(e0, st) != cudaSuccess) rc = fail(KW_ERR_CUDA, "autotune event");
        if (!rc) rc = batch_run(b, k, st, false);
        if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
          rc = fail(KW_ERR_CUDA, "autotune timing");
        if (!rc) rc = batch_reset(b);
        if (!rc && ms < best) {
          best = ms;
          bestT = Ts[ti];
          bestN = fr[fi][0];
          bestD = fr[fi][1];
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (kw_plan* p : b->plans) {
      set_generic_geometry(p, bestT, std::max(1, default_rows_per_block(p) * bestN / bestD));
      drop_graphs(p);
    }
    batch_clear(b);
    if (!rc) rc = batch_reset(b);
  }
  if (T_out) *T_out = bestT;
  if (R_num) *R_num = bestN;
  if (R_den) *R_den = bestD;
  return rc;
}

static int set_radix_order(kw_plan* p, int order) {
  for (int a = 0; a < p->D - 1; ++a)
    if (!factor_len(p->N[a], p->flen_axis[a], order)) return fail(KW_ERR_UNSUPPORTED, "radix schedule");
  if (!factor_len(p->Mfft, p->flen_row, order)) return fail(KW_ERR_UNSUPPORTED, "radix schedule");
  p->radix_order = order;
  drop_graphs(p);
  return KW_OK;
}

int32_t kw_plan_set_radix_order(kw_plan* p, int32_t order) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (order < 0 || order >= KW_RADIX_ORDERS) return fail(KW_ERR_INVALID, "radix schedule %d outside [0, %d)", order,
                                                          KW_RADIX_ORDERS);
  if (p->finalized) CK(cudaDeviceSynchronize());
  return set_radix_order(p, order);
}

int32_t kw_batch_set_radix_order(kw_batch* b, int32_t order) {
  if (!b) return fail(KW_ERR_INVALID, "null batch");
  if (order < 0 || order >= KW_RADIX_ORDERS) return fail(KW_ERR_INVALID, "radix schedule %d outside [0, %d)", order,
                                                          KW_RADIX_ORDERS);
  CK(cudaDeviceSynchronize());
  for (kw_plan* p : b->plans) {
    const int rc = set_radix_order(p, order);
    if (rc) return rc;
  }
  batch_clear(b);
  return KW_OK;
}

int32_t kw_batch_autotune_radix(kw_batch* b, int32_t nsteps, void* stream, int32_t* order_out) {
  if (!b) return fail(KW_ERR_INVALID, "null batch");
  for (kw_plan* p : b->plans)
    if (p->t != 0) return fail(KW_ERR_STATE, "kw_batch_autotune_radix needs every plan at t = 0");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int k = std::max(2, (int)nsteps);
  for (kw_plan* p : b->plans) k = std::min(k, p->g.Nt - 1);
  int best_order = b->plans.empty() ? 0 : b->plans[0]->radix_order;
  int rc = KW_OK;
  if (k >= 2) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int o = 0; o < KW_RADIX_ORDERS && !rc; ++o) {
      for (kw_plan* p : b->plans)
        if ((rc = set_radix_order(p, o))) break;
      if (rc) break;
      batch_clear(b);
      if ((rc = batch_run(b, 1 + k, st, false)) || (rc = batch_reset(b)) || (rc = batch_run(b, 1, st, false))) break;
      float ms = 0.f;
      if (cudaEventRecord(e0, st) != cudaSuccess) rc = fail(KW_ERR_CUDA, "autotune event");
      if (!rc) rc = batch_run(b, k, st, false);
      if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = fail(KW_ERR_CUDA, "autotune timing");
      if (!rc) rc = batch_reset(b);
      if (!rc && ms < best) {
        best = ms;
        best_order = o;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (kw_plan* p : b->plans) {
      const int r2 = set_radix_order(p, best_order);
      if (!rc) rc = r2;
    }
    batch_clear(b);
    if (!rc) rc = batch_reset(b);
  }
  if (order_out) *order_out = best_order;
  return rc;
}

int32_t kw_batch_set_loops(kw_batch* b, int32_t enable) {
  if (!b) return fail(KW_ERR_INVALID, "null batch");
  b->loops = enable != 0;
  return KW_OK;
}

int32_t kw_batch_graph_launches(const kw_batch* b, int64_t* count) {
  if (!b || !count) return fail(KW_ERR_INVALID, "kw_batch_graph_launches: null argument");
  *count = b->graph_launches;
  return KW_OK;
}

int32_t kw_batch_launch_count(const kw_batch* b, int64_t* count) {
  if (!b || !count) return fail(KW_ERR_INVALID, "null argument");
  long long c = b->launches;
  for (const kw_plan* p : b->plans) c += p->launches;
  *count = c;
  return KW_OK;
}

int32_t kw_batch_destroy(kw_batch* b) {
  if (!b) return KW_OK;
  cudaDeviceSynchronize();  // replays and side-stream work may still be in flight
  batch_free_graphs(b);
  if (b->d_loop) cudaFree(b->d_loop);
  if (b->cap) cudaStreamDestroy(b->cap);
  for (cudaStream_t x : b->side) cudaStreamDestroy(x);
  for (cudaEvent_t e : b->side_done) cudaEventDestroy(e);
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  for (void* a : b->allocs) cudaFree(a);
  delete b;
  return KW_OK;
}

static int check_device_error() {
  const int e = kw_device_error_take();
  if (e > 0) return fail(KW_ERR_CUDA, "a bounded device wait timed out (code %d); results of this run are invalid", e);
  if (e < 0) return fail(KW_ERR_CUDA, "could not read the device error word");
  return KW_OK;
}

int32_t kw_plan_sync(kw_plan* p, void* stream) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  CK(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)));
  return check_device_error();
}

int32_t kw_plan_time_index(const kw_plan* p, int32_t* t) {
  if (!p || !t) return fail(KW_ERR_INVALID, "null argument");
  *t = p->t;
  return KW_OK;
}

static int series_device(kw_plan* p, int series, float** out_dev, int* npts) {
  if (series < 0 || series > 6 || !p->d_rec[series]) return fail(KW_ERR_INVALID, "series %d was not recorded", series);
  const int np = p->interp_npts > 0 ? p->interp_npts : p->nslots;
  float* buf;
  int rc = dalloc(p, &buf, (size_t)np * p->nrec);
  if (rc) return rc;
  const long long tot = (long long)np * p->nrec;
  int grid = (int)std::min<long long>((tot + kThreads - 1) / kThreads, 65535);
  if (grid < 1) grid = 1;
  k_series_gather<<<grid, kThreads>>>(p->d_rec[series], p->nrec, p->nslots, np, p->interp_nc, p->d_islot, p->d_iw, buf);
  CK(cudaGetLastError());
  *out_dev = buf;
  *npts = np;
  return KW_OK;
}

static void dfree_last(kw_plan* p, void* ptr) {
  for (size_t i = 0; i < p->allocs.size(); ++i)
    if (p->allocs[i] == ptr) {
      cudaFree(ptr);
      p->allocs.erase(p->allocs.begin() + i);
      return;
    }
}

int32_t kw_plan_read_series(kw_plan* p, int32_t series, float* host, int64_t n) {
  if (!p || !host) return fail(KW_ERR_INVALID, "null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "plan not finalized");
  float* buf;
  int np;
  int rc = series_device(p, series, &buf, &np);
  if (rc) return rc;
  if (n != (long long)np * p->nrec) {
    dfree_last(p, buf);
    return fail(KW_ERR_INVALID, "series buffer has %lld values, expected %lld", (long long)n, (long long)np * p->nrec);
  }
  cudaError_t e = cudaMemcpy(host, buf, n * sizeof(float), cudaMemcpyDeviceToHost);
  dfree_last(p, buf);
  if (e != cudaSuccess) return fail(KW_ERR_CUDA, "read_series: %s", cudaGetErrorString(e));
  return KW_OK;
}

int32_t kw_plan_read_aggregate(kw_plan* p, int32_t series, int32_t kind, float* host, int64_t n) {
  if (!p || !host) return fail(KW_ERR_INVALID, "null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "plan not finalized");
  if (kind < 0 || kind > 2) return fail(KW_ERR_INVALID, "unknown aggregate %d", kind);
  float* buf;
  int np;
  int rc = series_device(p, series, &buf, &np);
  if (rc) return rc;
  if (n != np) {
    dfree_last(p, buf);
    return fail(KW_ERR_INVALID, "aggregate buffer has %lld values, expected %d", (long long)n, np);
  }
  float* agg;
  if ((rc = dalloc(p, &agg, np))) {
    dfree_last(p, buf);
    return rc;
  }
  k_series_reduce<<<(np + 255) / 256, 256>>>(buf, np, p->nrec, kind, agg);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(host, agg, n * sizeof(float), cudaMemcpyDeviceToHost);
  dfree_last(p, agg);
  dfree_last(p, buf);
  if (e != cudaSuccess) return fail(KW_ERR_CUDA, "read_aggregate: %s", cudaGetErrorString(e));
  return KW_OK;
}

static float* field_ptr(kw_plan* p, int field) {
  if (field == KW_FLD_P) return p->d_p;
  if (field >= KW_FLD_U0 && field <= KW_FLD_U2) return p->d_u[field - KW_FLD_U0];
  if (field >= KW_FLD_RHO0 && field <= KW_FLD_RHO2) return p->d_rho[field - KW_FLD_RHO0];
  return nullptr;
}

int32_t kw_plan_read_field(kw_plan* p, int32_t field, float* host, int64_t n) {
  if (!p || !host) return fail(KW_ERR_INVALID, "null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "plan not finalized");
  float* d = field_ptr(p, field);
  if (!d) return fail(KW_ERR_INVALID, "unknown field %d", field);
  if (n != p->ntot) return fail(KW_ERR_INVALID, "field buffer has %lld values, grid has %lld", (long long)n, p->ntot);
  CK(cudaMemcpy(host, d, n * sizeof(float), cudaMemcpyDeviceToHost));
  return KW_OK;
}

int32_t kw_plan_field_device_ptr(kw_plan* p, int32_t field, void** dptr) {
  if (!p || !dptr) return fail(KW_ERR_INVALID, "null argument");
  if (!p->finalized) return fail(KW_ERR_STATE, "plan not finalized");
  float* d = field_ptr(p, field);
  if (!d) return fail(KW_ERR_INVALID, "unknown field %d", field);
  *dptr = d;
  return KW_OK;
}

int32_t kw_plan_reset(kw_plan* p) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  if (!p->finalized) return fail(KW_ERR_STATE, "plan not finalized");
  CK(cudaDeviceSynchronize());
  int rc = zero_state(p);
  if (rc) return rc;
  CK(cudaDeviceSynchronize());
  p->t = 0;
  std::fill(p->ckpt_ok.begin(), p->ckpt_ok.end(), 0);
  return KW_OK;
}

int32_t kw_plan_set_timing(kw_plan* p, int32_t enable) {
  if (!p) return fail(KW_ERR_INVALID, "null plan");
  p->timing = enable != 0;
  p->ev_used.clear();
  p->ev_next = 0;
  return KW_OK;
}

int32_t kw_plan_read_timing(kw_plan* p, double* ms, int64_t* count) {
  if (!p || !ms || !count) return fail(KW_ERR_INVALID, "null argument");
  for (int c = 0; c < KW_K_NCLASS; ++c) {
    ms[c] = 0.0;
    count[c] = 0;
  }
  if (!p->ev_used.empty()) CK(cudaEventSynchronize(p->ev_pool[p->ev_used.back().second + 1]));
  for (auto& u : p->ev_used) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, p->ev_pool[u.second], p->ev_pool[u.second + 1]));
    if (u.first < 0 || u.first >= KW_K_NCLASS) continue;
    ms[u.first] += t;
    count[u.first] += 1;
  }
  return KW_OK;
}

int32_t kw_plan_launch_count(const kw_plan* p, int64_t* count) {
  if (!p || !count) return fail(KW_ERR_INVALID, "null argument");
  *count = p->launches;
  return KW_OK;
}

int32_t kw_plan_destroy(kw_plan* p) {
  if (!p) return KW_OK;
  cudaDeviceSynchronize();  // graph replays may still read the plan's buffers
  for (cudaEvent_t e : p->ev_pool) cudaEventDestroy(e);
  drop_graphs(p);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->tma) kw_tma_plan_destroy(p->tma);
  for (void* a : p->allocs) cudaFree(a);
  delete p;
  return KW_OK;
}

}  // extern "C"
