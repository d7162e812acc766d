// Library runtime: error reporting, device selection, device workspaces.
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "ctr_internal.h"

namespace ctr {

static thread_local char g_last_error[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  return e == cudaErrorMemoryAllocation ? CTR_ERR_ALLOC : CTR_ERR_CUDA;
}

// Device workspaces.  The buffers grow geometrically and are only freed by
// ctr_release_workspace(); a call that needs more scratch synchronises the
// device first, so a buffer is never freed while kernels still read it.
static Workspace g_ws[WS_COUNT];
static std::mutex g_ws_mutex;

int Workspace::get(size_t need, void** out) {
  if (need == 0) need = 256;
  if (need > bytes) {
    size_t nb = bytes ? bytes : (size_t)1 << 20;
    while (nb < need) nb *= 2;
    if (ptr) {
      CTR_CUDA(cudaDeviceSynchronize());
      CTR_CUDA(cudaFree(ptr));
      ptr = nullptr;
      bytes = 0;
    }
    cudaError_t e = cudaMalloc(&ptr, nb);
    if (e != cudaSuccess) {
      // retry with the exact size before giving up
      cudaGetLastError();
      e = cudaMalloc(&ptr, need);
      if (e != cudaSuccess) {
        ptr = nullptr;
        return cuda_fail(e, "cudaMalloc(workspace)", __FILE__, __LINE__);
      }
      nb = need;
    }
    bytes = nb;
  }
  *out = ptr;
  return CTR_OK;
}

void Workspace::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

Workspace& workspace(int slot) { return g_ws[slot]; }

// Host-to-device upload through a mapped pinned staging buffer per slot: a small
// kernel reads the staging buffer over the host link and writes the device
// workspace, so the tables of a call never queue behind large copy-engine
// transfers that a caller runs on other streams (e.g. the next step's inputs),
// and the caller's host array may be reused at once.
struct Staging {
  void* host = nullptr;
  void* host_dev = nullptr;  // device alias of the mapped staging buffer
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
};
static Staging g_stage[WS_COUNT];

int upload(int slot, const void* host, size_t bytes, void** dev, cudaStream_t stream) {
  Staging& s = g_stage[slot];
  if (s.done) CTR_CUDA(cudaEventSynchronize(s.done));  // the previous upload from this buffer was consumed
  if (bytes > s.bytes) {
    if (s.host) CTR_CUDA(cudaFreeHost(s.host));
    s.host = nullptr;
    size_t nb = bytes < 4096 ? 4096 : bytes * 2;
    CTR_CUDA(cudaHostAlloc(&s.host, nb, cudaHostAllocMapped));
    CTR_CUDA(cudaHostGetDevicePointer(&s.host_dev, s.host, 0));
    s.bytes = nb;
  }
  if (!s.done) CTR_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
  std::memcpy(s.host, host, bytes);
  CTR_TRY(g_ws[slot].get(bytes, dev));
  CTR_TRY(launch_stage_copy(*dev, s.host_dev, bytes, stream));
  CTR_CUDA(cudaEventRecord(s.done, stream));
  return CTR_OK;
}

// ---------------------------------------------------------- kernel timing
// Every kernel launch of the library goes through TimedLaunch.  Launches are
// always counted per kernel name; when timing is enabled, a CUDA event pair is
// recorded on the launching stream around each launch, so per-kernel device
// durations can be read back after the timed region (ctr_timing_report).
struct TimingRec {
  const char* name;
  int ev;  // index of the start event in the pool (stop = ev + 1)
};
static std::mutex g_tm_mutex;
static bool g_timing = false;
static std::vector<TimingRec> g_trec;
static std::vector<cudaEvent_t> g_pool;
static std::vector<std::pair<const char*, long long>> g_counts;

static void count_launch(const char* name) {
  for (auto& c : g_counts)
    if (c.first == name || std::strcmp(c.first, name) == 0) {
      c.second++;
      return;
    }
  g_counts.emplace_back(name, 1);
}

TimedLaunch::TimedLaunch(cudaStream_t s, const char* name) : stream_(s), idx_(-1) {
  std::lock_guard<std::mutex> lk(g_tm_mutex);
  count_launch(name);
  if (!g_timing) return;
  int ev = (int)g_trec.size() * 2;
  while ((int)g_pool.size() < ev + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    g_pool.push_back(e);
  }
  g_trec.push_back(TimingRec{name, ev});
  idx_ = ev;
  cudaEventRecord(g_pool[ev], s);
}

TimedLaunch::~TimedLaunch() {
  if (idx_ < 0) return;
  std::lock_guard<std::mutex> lk(g_tm_mutex);
  cudaEventRecord(g_pool[idx_ + 1], stream_);
}

}  // namespace ctr

extern "C" {

void ctr_timing_enable(int on) {
  std::lock_guard<std::mutex> lk(ctr::g_tm_mutex);
  ctr::g_timing = on != 0;
  ctr::g_trec.clear();
  ctr::g_counts.clear();
}

long long ctr_launch_count(void) {
  std::lock_guard<std::mutex> lk(ctr::g_tm_mutex);
  long long n = 0;
  for (auto& c : ctr::g_counts) n += c.second;
  return n;
}

int ctr_timing_report(char* buf, int buflen) {
  std::lock_guard<std::mutex> lk(ctr::g_tm_mutex);
  if (!buf || buflen < 3) return ctr::fail(CTR_ERR_ARG, "ctr_timing_report: buffer too small");
  std::vector<std::pair<const char*, std::pair<long long, double>>> agg;
  for (auto& r : ctr::g_trec) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(ctr::g_pool[r.ev + 1]);
    if (e != cudaSuccess) return ctr::cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__);
    CTR_CUDA(cudaEventElapsedTime(&ms, ctr::g_pool[r.ev], ctr::g_pool[r.ev + 1]));
    bool found = false;
    for (auto& a : agg)
      if (std::strcmp(a.first, r.name) == 0) {
        a.second.first++;
        a.second.second += ms;
        found = true;
      }
    if (!found) agg.push_back({r.name, {1, (double)ms}});
  }
  std::string s = "{";
  for (size_t i = 0; i < ctr::g_counts.size(); i++) {
    const char* name = ctr::g_counts[i].first;
    double ms = 0.0;
    long long timed = 0;
    for (auto& a : agg)
      if (std::strcmp(a.first, name) == 0) timed = a.second.first, ms = a.second.second;
    char item[256];
    snprintf(item, sizeof(item), "%s\"%s\": [%lld, %lld, %.6f]", i ? ", " : "", name, ctr::g_counts[i].second,
             timed, ms);
    s += item;
  }
  s += "}";
  if ((int)s.size() + 1 > buflen) return ctr::fail(CTR_ERR_ARG, "ctr_timing_report: buffer too small");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return CTR_OK;
}

int ctr_version(void) { return 100; }

const char* ctr_error_string(int code) {
  switch (code) {
    case CTR_OK: return "ok";
    case CTR_ERR_ARG: return "invalid argument";
    case CTR_ERR_CUDA: return "CUDA error";
    case CTR_ERR_ALLOC: return "allocation failed";
    case CTR_ERR_UNSUPPORTED: return "unsupported device or feature";
    case CTR_ERR_TIMEOUT: return "device-side wait timed out";
    case CTR_ERR_IO: return "I/O error";
    default: return "unknown error";
  }
}

const char* ctr_last_error(void) { return ctr::g_last_error; }

int ctr_device_init(int device) {
  int count = 0;
  CTR_CUDA(cudaGetDeviceCount(&count));
  if (count == 0) return ctr::fail(CTR_ERR_UNSUPPORTED, "no CUDA device found");
  if (device < 0 || device >= count) return ctr::fail(CTR_ERR_ARG, "device id %d not in [0,%d)", device, count);
  CTR_CUDA(cudaSetDevice(device));
  cudaDeviceProp p;
  CTR_CUDA(cudaGetDeviceProperties(&p, device));
  if (p.major != 10 || p.minor != 3)
    return ctr::fail(CTR_ERR_UNSUPPORTED, "device %d is sm_%d%d; this build targets sm_103 (GB300)", device,
                     p.major, p.minor);
  return CTR_OK;
}

void ctr_release_workspace(void) {
  std::lock_guard<std::mutex> lk(ctr::g_ws_mutex);
  cudaDeviceSynchronize();
  for (int i = 0; i < ctr::WS_COUNT; i++) ctr::g_ws[i].release();
}

}  // extern "C"
