// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "ctr.h"

namespace ctr {

// ----------------------------------------------------------- error handling
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define CTR_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::ctr::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define CTR_TRY(call)              \
  do {                             \
    int _rc = (call);              \
    if (_rc != CTR_OK) return _rc; \
  } while (0)

// Counts (and, when enabled, times with CUDA events) one kernel launch, and
// marks it with an NVTX range of the kernel's name for timeline profilers.
class TimedLaunch {
 public:
  TimedLaunch(cudaStream_t s, const char* name);
  ~TimedLaunch();

 private:
  cudaStream_t stream_;
  int idx_;
  bool ranged_ = false;
};

// --------------------------------------------------------------- tables
struct Tables {
  int16_t rho_spin[768][4];
  int16_t rho_lprp[768][2];
  float rho_coef[768][2];
  int16_t rhopi_spin[768][6];
  int16_t rhopi_ip[768];
  float rhopi_coef[768][2];
  int16_t sq_spin[256][6];
  float sq_coef[256][2];
  int16_t dt_spin[256][6];
  float dt_coef[256][2];
  int16_t dth_spin[256][4];
  float dth_coef[256][2];
  int16_t sigma_spin[64][4];
  int16_t sigma_lprp[64][2];
  float sigma_coef[64][2];
  int16_t hf_spin[16][2];
  float hf_coef[16][2];
  int16_t tri_spin[128][5];
  int16_t tri_ip[128];
  float tri_coef[128][2];
};
const Tables& tables();

// ------------------------------------------------------------ workspace
// Device scratch owned by the library: one growable buffer per purpose,
// reused across calls (every call on one stream uses it in order).
struct Workspace {
  void* ptr = nullptr;
  size_t bytes = 0;
  int get(size_t need, void** out);
  void release();
};
Workspace& workspace(int slot);
enum {
  WS_SCRATCH = 0,   // per-batch products / sliced operands
  WS_TASKS,         // uploaded task lists (several independent slots)
  WS_TASKS2,
  WS_GEMM_A,
  WS_GEMM_B,
  WS_ROWTASKS,
  WS_ROWS,          // per-row partial results
  WS_PHI,           // sliced elementals
  WS_MISC,          // small tables (CSR of output rows)
  WS_ROWABS,        // per-row error scales of the split engine
  WS_REFINE,        // refinement list / patches of the split engine
  WS_SPLITTASK,     // sliced operands of split-engine task stages
  WS_SPLITJOBS,     // their job / instance / pointer tables
  WS_SPLITJOBS2,
  WS_SPLITJOBS3,
  WS_RPHI,          // per-time-slice products of a recomputation call
  WS_SPLITJOBS4,    // distinct blocks of a task launch
  WS_BLOCKEXP,      // their row / column exponent bounds
  WS_TRACEGROUPS,   // grouped closing traces of a two-sided call
  WS_GRAM,          // sliced operands and partial products of Gram traces
  WS_GRAMJOBS,      // their block, instance and pointer tables
  WS_GRAMTRACES,    // their trace lists
  WS_COUNT
};

// Perambulator file payload (complex128, file order) -> host buffer in the library layout.
int reorder_prop_device(int N, int Nt, const double* file_payload, int single, void* host_out);

// Per-entry accuracy control of the split engine (ctr_split_set_refine): relative
// tolerance (0 = off) and the number of entries the last split call recomputed.
extern double g_refine_tol;
extern long long g_refined_last;
// Work of the split engine's launches since the last reset (ctr_split_flops): BF16
// MMA flops the tensor cores executed (padding included) and the Nev x Nev complex
// block products they computed (8 Nev^3 FP64-equivalent flops each).  Counted by
// eager launches; replays of recorded graphs are not counted.
extern double g_split_mma_flops, g_split_products;
// The same for the Gram products of closing traces (ctr_gram_flops): executed
// BF16 MMA flops and the traces they produced (8 Nev^2 FP64-equivalent flops each).
extern double g_gram_mma_flops, g_gram_traces;

// Reads (and clears) the device-side error flag of the split engine; syncs the stream.
int split_error_check(cudaStream_t s);
// Runs a bounded device wait that times out after timeout_ms and reports it (ctr_wait_probe).
int wait_probe(int timeout_ms, cudaStream_t s);
// The split GEMM's MMA schedule alone (ctr_mma_schedule_probe).
int mma_schedule_probe(int hp, int nchunk, double* clocks_per_mma, double* tflops, cudaStream_t s);
int zgemm_split_batched(int N, int nb, const double* const* x, const double* const* y, double* const* c,
                        cudaStream_t stream);
// A stage of FP64-engine GEMM tasks (struct ZTask, kernels.h) on the split
// engine: C = sum_q w_q op(A_q) op(B_q) with real power-of-two weights.
struct ZTask;
int zgemm_split_tasks(int N, const ZTask* tasks, int ntask, cudaStream_t stream);

// A grid of block products that share their right side:
//   C(s, j) = sum_{q < nterm} w_q op(A[s * nterm + q]) op(B[j][q]),  s < nslab, j < nb <= 8,
// written at C0[j] + s * Nev^2 (the slabs' outputs of one right block are
// consecutive blocks).  op: conjugate transpose where bit q of adag / bit 4j+q of
// bdag is set.  On the split engine the slabs stack along M, so that 128-row
// tiles carry no padding rows between them; weights must be real powers of two.
struct GridTask {
  std::vector<const double2*> A;
  const double2* B[8][4];
  double2* C0[8];
  float w[4];
  int nslab, nb, nterm, adag, bdag;
};
int zgemm_split_grids(int N, const std::vector<GridTask>& grids, cudaStream_t stream);

// Closing traces Tr-Had(X, Y) = sum_e X_e conj(Y_e) of many left and right
// blocks that meet in groups, as Gram products on the split engine: group g has
// left blocks left[g * mrows + r] and right blocks right[g * ncols + c] (null:
// a block of zeros); trace k of tr takes (g, r, c) and writes coef * value to
// trv[slot] and, where tra is not null, its error scale to tra[slot] (a bound of
// sum |X|_1 |Y|_1 and of the slices' truncation, relative to which the value
// keeps ~2^-52).
struct GramPlan {
  struct Tr {
    int g, r, c, slot;
    float cre, cim;
  };
  int ngroup = 0, mrows = 0, ncols = 0;
  // groups come in runs of group_run whose traces may interleave in tr, runs in
  // order: a launch then takes whole runs, and its traces are one range of tr
  int group_run = 1;
  std::vector<const double2*> left, right;
  std::vector<Tr> tr;
};
int trace_gram(int N, const GramPlan& plan, double2* trv, double* tra, cudaStream_t stream);

// ------------------------------------------------------------ graph capture
// A host step that reads device results (e.g. the split engine's refinement
// list).  Run at once by eager calls; while the thread records a graph, it ends
// the current graph segment and runs after that segment at every launch, on the
// launch stream.  Steps capture what they need by value.
using HostStep = std::function<int(cudaStream_t)>;
int host_step(cudaStream_t s, HostStep fn);
bool capturing();
#define CTR_NO_CAPTURE(name)                                                                         \
  do {                                                                                               \
    if (::ctr::capturing())                                                                          \
      return ::ctr::fail(CTR_ERR_UNSUPPORTED, "%s reads device data on the host to plan its work and " \
                         "cannot be recorded into a graph", name);                                   \
  } while (0)
// One-time device state needed before a capture (error flag, kernel attributes).
int prepare_for_capture();

// ---------------------------------------------------------------- autotuner
// Knob choices keyed by "knob|shape" (tune.cpp).  tune_mode() is 0 while the
// thread records a graph.  tune_resolve returns the forced value, the cached
// choice, a fresh measurement of run(c) for c < ncand (mode >= 1), or dflt.
int tune_mode();
std::string tune_key(const char* knob, const std::string& shape);
int tune_forced(const char* knob);
bool tune_lookup(const std::string& key, int* choice);
void tune_store(const std::string& key, int choice, const std::vector<double>& ms);
int tune_resolve(const char* knob, const std::string& shape, int ncand, int dflt, cudaStream_t s,
                 const std::function<int(int)>& run, int* choice);
// The choice tune_resolve will return when it will not measure (forced, cached or
// mode 0): true and *choice set; false when it would measure the candidates.
bool tune_peek(const char* knob, const std::string& shape, int ncand, int dflt, int* choice);

// Upload a host array into a workspace slot (async on stream, host buffer is
// kept alive by a pinned staging copy owned by the slot).
int upload(int slot, const void* host, size_t bytes, void** dev, cudaStream_t stream);
// Several host arrays in one upload (one staging copy): devs[i] receives the
// device address of parts[i] (256-byte aligned inside the slot).
int upload_group(int slot, const std::vector<std::pair<const void*, size_t>>& parts, void** devs,
                 cudaStream_t stream);
// dst (device) <- src (device-accessible, e.g. mapped pinned host memory), by a kernel.
int launch_stage_copy(void* dst, const void* src, size_t bytes, cudaStream_t stream);
// dst <- src for any alignment (a kernel; dst may be mapped pinned host memory).
int launch_readback(void* dst, const void* src, size_t bytes, cudaStream_t stream);
// Reads a small device result into host memory through a mapped pinned buffer
// written by a kernel (never queued behind copy-engine transfers that a caller
// runs on other streams); synchronises the stream.  Not usable while recording.
int download(void* host, const void* dev, size_t bytes, cudaStream_t stream);

// ------------------------------------------------------- two-sided plan
struct TwoSidedRow {
  int16_t a, b, c, d, L, R;  // sink block (a,b) with Phi_R(tf); source block (c,d) with Phi_L(ti)
};

int twosided_fp64(int nev, int nt, int tf_begin, int tf_end, const double* prop_rows, const double* phi,
                  int nphi, const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                  const std::vector<int32_t>& out_index, int nout, double* out, cudaStream_t stream);
int twosided_split(int nev, int nt, int tf_begin, int tf_end, const double* prop_rows, const double* phi,
                   int nphi, const std::vector<TwoSidedRow>& rows, const std::vector<float>& coef,
                   const std::vector<int32_t>& out_index, int nout, double* out, cudaStream_t stream);

// Traces of chains of perambulator blocks and plain elementals (the chain
// program of the profile adjoint, without a profile): values[c] = Tr[F_1 ... F_n]
// for chain c = factors[off[c] .. off[c+1]); perambulator factors index prop
// [rows][Nt][4][4][N][N] by (a = row, b = t2).  engine: where the products run
// (CTR_ENGINE_SPLIT: the high-precision split configuration); traces are FP64.
int chain_values(int N, int Nt, int nphi, const double* prop, const double* phi, const std::vector<ctr_factor>& factors,
                 const std::vector<int>& off, double* values, cudaStream_t s, int engine);

// ------------------------------------------- reference-compatible C++ layer
// State set by initContract (api.cu): false while the library is off.
bool contract_state(int* nev, int* nt);
// The reference's result text blocks (the dumpData bodies of lib/contract.cpp),
// appended to f from source-averaged correlators [Nt][ncorr] complex (interleaved
// re/im doubles); loop and fish_hor take the per-time values [Nt].
void dump_rho(FILE* f, const double* avg, int nt);
void dump_rhopi(FILE* f, const double* avg, int nt);
void dump_pipi(FILE* f, const double* avg, int nt, int isospin);
void dump_loop(FILE* f, const double* loop, int nt);
void dump_sigma(FILE* f, const double* avg, int nt);
void dump_fish_hor(FILE* f, const double* hf, int nt);
void dump_triangle(FILE* f, const double* avg, int nt);
// Frees the device staging buffers of the texture-object launchers (compat.cu).
void compat_release();

}  // namespace ctr
