// Library runtime: error reporting, device selection, device workspaces.
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <mutex>

#include <nvtx3/nvToolsExt.h>

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

// ------------------------------------------------------------ graph capture
// While a thread records (ctr_graph_begin .. ctr_graph_end), the library's
// scratch requests, table uploads and launches are redirected here: scratch and
// tables live in device memory owned by the recording, tables are copied once
// on a private stream, and kernels land in the captured graph.
struct Segment {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t kernels = 0;
  std::vector<HostStep> tails;  // host steps that follow this segment
};

}  // namespace ctr

struct ctr_graph {
  cudaStream_t stream = nullptr;
  cudaStream_t setup = nullptr;  // non-capturing stream for the one-time table copies
  std::vector<ctr::Segment> segs;
  std::vector<void*> blocks;     // device memory owned by the graph
  size_t block_bytes = 0;
  void* ws_ptr[ctr::WS_COUNT] = {};
  size_t ws_bytes[ctr::WS_COUNT] = {};
  uint8_t* arena = nullptr;
  size_t arena_used = 0, arena_cap = 0;
  std::vector<std::pair<const char*, long long>> counts;  // kernel launches per replay
  int error = CTR_OK;
};

namespace ctr {

static thread_local ctr_graph* g_cap = nullptr;

bool capturing() { return g_cap != nullptr; }

// Allocations while the thread captures are "potentially unsafe" calls: they
// are made in relaxed capture mode for the thread, as CUDA documents for
// allocators used under capture.
struct RelaxedCapture {
  cudaStreamCaptureMode mode = cudaStreamCaptureModeRelaxed;
  RelaxedCapture() { cudaThreadExchangeStreamCaptureMode(&mode); }
  ~RelaxedCapture() { cudaThreadExchangeStreamCaptureMode(&mode); }
};

static int graph_alloc(ctr_graph& g, size_t bytes, void** out) {
  void* p = nullptr;
  cudaError_t e;
  {
    RelaxedCapture rc;
    e = cudaMalloc(&p, bytes);
  }
  if (e != cudaSuccess) {
    g.error = CTR_ERR_ALLOC;
    return cuda_fail(e, "cudaMalloc(graph memory)", __FILE__, __LINE__);
  }
  g.blocks.push_back(p);
  g.block_bytes += bytes;
  *out = p;
  return CTR_OK;
}

static int capture_workspace(int slot, size_t need, void** out) {
  ctr_graph& g = *g_cap;
  if (need == 0) need = 256;
  if (g.ws_bytes[slot] < need) {
    // earlier nodes of the recording keep the smaller buffer: it stays owned
    CTR_TRY(graph_alloc(g, need, &g.ws_ptr[slot]));
    g.ws_bytes[slot] = need;
  }
  *out = g.ws_ptr[slot];
  return CTR_OK;
}

static int capture_upload(const void* host, size_t bytes, void** dev) {
  ctr_graph& g = *g_cap;
  const size_t nb = (bytes + 255) & ~(size_t)255;
  if (g.arena_used + nb > g.arena_cap) {
    const size_t cap = std::max(nb, (size_t)16 << 20);
    void* p;
    CTR_TRY(graph_alloc(g, cap, &p));
    g.arena = (uint8_t*)p;
    g.arena_used = 0;
    g.arena_cap = cap;
  }
  void* dst = g.arena + g.arena_used;
  g.arena_used += nb;
  if (bytes) {
    RelaxedCapture rc;
    cudaError_t e = cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, g.setup);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g.setup);
    if (e != cudaSuccess) {
      g.error = CTR_ERR_CUDA;
      return cuda_fail(e, "table copy while recording", __FILE__, __LINE__);
    }
  }
  *dev = dst;
  return CTR_OK;
}

static int close_segment(ctr_graph& g) {
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(g.stream, &graph);
  if (e != cudaSuccess || !graph) {
    g.error = CTR_ERR_CUDA;
    return cuda_fail(e != cudaSuccess ? e : cudaErrorStreamCaptureInvalidated, "cudaStreamEndCapture", __FILE__,
                     __LINE__);
  }
  Segment sg;
  sg.graph = graph;
  size_t n = 0;
  CTR_CUDA(cudaGraphGetNodes(graph, nullptr, &n));
  if (n) {
    std::vector<cudaGraphNode_t> nodes(n);
    CTR_CUDA(cudaGraphGetNodes(graph, nodes.data(), &n));
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      CTR_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t == cudaGraphNodeTypeKernel) sg.kernels++;
    }
  }
  g.segs.push_back(std::move(sg));
  return CTR_OK;
}

static int open_segment(ctr_graph& g) {
  CTR_CUDA(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
  return CTR_OK;
}

int host_step(cudaStream_t s, HostStep fn) {
  if (!g_cap) return fn(s);
  ctr_graph& g = *g_cap;
  if (s != g.stream) {
    g.error = CTR_ERR_ARG;
    return fail(CTR_ERR_ARG, "call on a stream other than the recording one");
  }
  CTR_TRY(close_segment(g));
  g.segs.back().tails.push_back(std::move(fn));
  return open_segment(g);
}

static void destroy_graph(ctr_graph* g) {
  if (!g) return;
  for (auto& sg : g->segs) {
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    if (sg.graph) cudaGraphDestroy(sg.graph);
  }
  if (!g->blocks.empty()) cudaDeviceSynchronize();
  for (void* p : g->blocks) cudaFree(p);
  if (g->setup) cudaStreamDestroy(g->setup);
  delete g;
}

// Device workspaces.  The buffers grow geometrically and are only freed by
// ctr_release_workspace(); a call that needs more scratch synchronises the
// device first, so a buffer is never freed while kernels still read it.
static Workspace g_ws[WS_COUNT];
static std::mutex g_ws_mutex;

int Workspace::get(size_t need, void** out) {
  if (g_cap) return capture_workspace((int)(this - g_ws), need, out);
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
  if (g_cap) return capture_upload(host, bytes, dev);
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

int upload_group(int slot, const std::vector<std::pair<const void*, size_t>>& parts, void** devs,
                 cudaStream_t stream) {
  std::vector<size_t> off(parts.size());
  size_t total = 0;
  for (size_t i = 0; i < parts.size(); i++) {
    off[i] = total;
    total += (parts[i].second + 255) & ~(size_t)255;
  }
  std::vector<uint8_t> packed(std::max<size_t>(total, 1));
  for (size_t i = 0; i < parts.size(); i++)
    if (parts[i].second) std::memcpy(packed.data() + off[i], parts[i].first, parts[i].second);
  void* d;
  CTR_TRY(upload(slot, packed.data(), total, &d, stream));
  for (size_t i = 0; i < parts.size(); i++) devs[i] = (uint8_t*)d + off[i];
  return CTR_OK;
}

static std::mutex g_down_mutex;
static void* g_down_host = nullptr;
static void* g_down_dev = nullptr;
static size_t g_down_bytes = 0;

int download(void* host, const void* dev, size_t bytes, cudaStream_t stream) {
  if (g_cap) return fail(CTR_ERR_UNSUPPORTED, "device results cannot be read while recording a graph");
  if (bytes == 0) return CTR_OK;
  std::lock_guard<std::mutex> lk(g_down_mutex);
  if (bytes > g_down_bytes) {
    if (g_down_host) CTR_CUDA(cudaFreeHost(g_down_host));
    g_down_host = nullptr;
    g_down_bytes = 0;
    const size_t nb = std::max<size_t>(bytes * 2, 4096);
    CTR_CUDA(cudaHostAlloc(&g_down_host, nb, cudaHostAllocMapped));
    CTR_CUDA(cudaHostGetDevicePointer(&g_down_dev, g_down_host, 0));
    g_down_bytes = nb;
  }
  CTR_TRY(launch_readback(g_down_dev, dev, bytes, stream));
  CTR_CUDA(cudaStreamSynchronize(stream));
  std::memcpy(host, g_down_host, bytes);
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

static void count_into(std::vector<std::pair<const char*, long long>>& v, const char* name, long long n);
static void count_launch(const char* name) { count_into(g_counts, name, 1); }

static void count_into(std::vector<std::pair<const char*, long long>>& v, const char* name, long long n) {
  for (auto& c : v)
    if (c.first == name || std::strcmp(c.first, name) == 0) {
      c.second += n;
      return;
    }
  v.emplace_back(name, n);
}

TimedLaunch::TimedLaunch(cudaStream_t s, const char* name) : stream_(s), idx_(-1) {
  if (g_cap) {
    // recorded, not executed: counted per replay by ctr_graph_launch
    count_into(g_cap->counts, name, 1);
    if (s != g_cap->stream) {
      g_cap->error = CTR_ERR_ARG;
      set_error("%s launched on a stream other than the recording one", name);
    }
    return;
  }
  nvtxRangePushA(name);
  ranged_ = true;
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
  if (idx_ >= 0) {
    std::lock_guard<std::mutex> lk(g_tm_mutex);
    cudaEventRecord(g_pool[idx_ + 1], stream_);
  }
  if (ranged_) nvtxRangePop();
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
  if (ctr::capturing()) return;  // recorded graphs own their scratch; eager buffers stay until after recording
  std::lock_guard<std::mutex> lk(ctr::g_ws_mutex);
  cudaDeviceSynchronize();
  for (int i = 0; i < ctr::WS_COUNT; i++) ctr::g_ws[i].release();
}

int ctr_graph_begin(void* stream) {
  using namespace ctr;
  if (g_cap) return fail(CTR_ERR_ARG, "ctr_graph_begin: this thread is already recording");
  cudaStream_t s = (cudaStream_t)stream;
  if (!s || s == cudaStreamLegacy || s == cudaStreamPerThread)
    return fail(CTR_ERR_ARG, "ctr_graph_begin: recording needs a created stream, not a default stream");
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  CTR_CUDA(cudaStreamIsCapturing(s, &st));
  if (st != cudaStreamCaptureStatusNone) return fail(CTR_ERR_ARG, "ctr_graph_begin: the stream is already capturing");
  // one-time device state (error flag, kernel attributes) is set up before capture
  CTR_TRY(prepare_for_capture());
  ctr_graph* g = new ctr_graph;
  g->stream = s;
  cudaError_t e = cudaStreamCreateWithFlags(&g->setup, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "cudaStreamCreateWithFlags", __FILE__, __LINE__);
  }
  int rc = open_segment(*g);
  if (rc != CTR_OK) {
    destroy_graph(g);
    return rc;
  }
  g_cap = g;
  return CTR_OK;
}

int ctr_graph_end(void* stream, ctr_graph** out) {
  using namespace ctr;
  if (out) *out = nullptr;
  if (!g_cap) return fail(CTR_ERR_ARG, "ctr_graph_end: this thread is not recording");
  ctr_graph* g = g_cap;
  g_cap = nullptr;
  const int prior = g->error;
  const std::string prior_msg = ctr_last_error();
  int rc = close_segment(*g);
  if (rc == CTR_OK && prior != CTR_OK) {
    rc = prior;
    set_error("ctr_graph_end: a call failed while recording: %s", prior_msg.c_str());
  }
  if (rc == CTR_OK && (cudaStream_t)stream != g->stream)
    rc = fail(CTR_ERR_ARG, "ctr_graph_end: stream differs from the one passed to ctr_graph_begin");
  if (rc == CTR_OK && !out) rc = fail(CTR_ERR_ARG, "ctr_graph_end: null output");
  for (size_t i = 0; rc == CTR_OK && i < g->segs.size(); i++) {
    Segment& sg = g->segs[i];
    size_t n = 0;
    cudaError_t e = cudaGraphGetNodes(sg.graph, nullptr, &n);
    if (e == cudaSuccess && n) e = cudaGraphInstantiate(&sg.exec, sg.graph, 0);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
  }
  if (rc != CTR_OK) {
    destroy_graph(g);
    return rc;
  }
  *out = g;
  return CTR_OK;
}

int ctr_graph_launch(ctr_graph* g, void* stream) {
  using namespace ctr;
  if (!g) return fail(CTR_ERR_ARG, "ctr_graph_launch: null graph");
  if (g_cap) return fail(CTR_ERR_ARG, "ctr_graph_launch: not available while this thread records");
  cudaStream_t s = (cudaStream_t)stream;
  g_refined_last = 0;
  for (auto& sg : g->segs) {
    if (sg.exec) CTR_CUDA(cudaGraphLaunch(sg.exec, s));
    for (auto& t : sg.tails) CTR_TRY(t(s));
  }
  std::lock_guard<std::mutex> lk(g_tm_mutex);
  for (auto& c : g->counts) count_into(g_counts, c.first, c.second);
  return CTR_OK;
}

int ctr_graph_info(const ctr_graph* g, int* nsegments, long long* nkernels, long long* device_bytes) {
  if (!g) return ctr::fail(CTR_ERR_ARG, "ctr_graph_info: null graph");
  long long k = 0;
  for (auto& sg : g->segs) k += (long long)sg.kernels;
  if (nsegments) *nsegments = (int)g->segs.size();
  if (nkernels) *nkernels = k;
  if (device_bytes) *device_bytes = (long long)g->block_bytes;
  return CTR_OK;
}

void ctr_graph_destroy(ctr_graph* g) { ctr::destroy_graph(g); }

}  // extern "C"
