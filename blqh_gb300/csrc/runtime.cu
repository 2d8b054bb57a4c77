// Context, errors, device memory, kernel-class timers and a device scan.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "blqh_internal.h"

static thread_local std::string g_thread_error;

void set_error(blqh_ctx* ctx, int code, const std::string& msg) {
  (void)code;
  g_thread_error = msg;
  if (ctx) ctx->last_error = msg;
}

// ---------------------------------------------------------------------------
// Device memory: a caching allocator. cudaFree synchronizes the whole device
// and cudaMalloc costs tens of microseconds, which dominated setting up many
// small sectors (a batched sweep builds thousands). Blocks are rounded up to a
// bucket size and, when freed, kept per context with an event recorded on the
// context's stream; a later allocation of the same bucket takes the block
// after that event has completed (the work that used it is done), so the
// block can be written from any stream or from the host. Cached bytes are
// capped; an allocation that fails empties the cache and retries once.
namespace {
struct Live {
  size_t bytes;
  blqh_ctx* ctx;
};
struct Cached {
  void* p;
  cudaEvent_t ev;
};
std::mutex g_mem_mu;
std::unordered_map<void*, Live> g_live;
std::map<std::pair<blqh_ctx*, size_t>, std::vector<Cached>> g_cache;
size_t g_cached_bytes = 0;
const size_t kCacheCap = (size_t)16 << 30;

size_t bucket_bytes(size_t b) {
  if (b < 512) return 512;
  if (b <= ((size_t)1 << 20)) {
    size_t v = 512;
    while (v < b) v <<= 1;
    return v;
  }
  const size_t g = (size_t)2 << 20;
  return (b + g - 1) / g * g;
}

void release_cached(blqh_ctx* only) {
  // caller holds g_mem_mu
  for (auto it = g_cache.begin(); it != g_cache.end();) {
    if (only && it->first.first != only) {
      ++it;
      continue;
    }
    for (auto& c : it->second) {
      cudaEventSynchronize(c.ev);
      cudaEventDestroy(c.ev);
      cudaFree(c.p);
      g_cached_bytes -= it->first.second;
    }
    it = g_cache.erase(it);
  }
}
}  // namespace

void* dev_alloc(blqh_ctx* ctx, size_t bytes) {
  const size_t b = bucket_bytes(bytes);
  {
    std::lock_guard<std::mutex> lk(g_mem_mu);
    auto it = g_cache.find({ctx, b});
    if (it != g_cache.end() && !it->second.empty()) {
      Cached c = it->second.back();
      it->second.pop_back();
      g_cached_bytes -= b;
      cudaEventSynchronize(c.ev);
      cudaEventDestroy(c.ev);
      g_live[c.p] = Live{b, ctx};
      return c.p;
    }
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, b);
  if (e != cudaSuccess) {
    cudaGetLastError();
    {
      std::lock_guard<std::mutex> lk(g_mem_mu);
      release_cached(nullptr);
    }
    e = cudaMalloc(&p, b);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(ctx, BLQH_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
                                       cudaGetErrorString(e));
    throw BlqhError{BLQH_ERR_NOMEM, "cudaMalloc"};
  }
  std::lock_guard<std::mutex> lk(g_mem_mu);
  g_live[p] = Live{b, ctx};
  return p;
}

void dev_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_mem_mu);
  auto it = g_live.find(p);
  if (it == g_live.end()) {
    cudaFree(p);
    return;
  }
  const Live l = it->second;
  g_live.erase(it);
  cudaEvent_t ev = nullptr;
  if (!l.ctx || g_cached_bytes + l.bytes > kCacheCap ||
      cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ev, l.ctx->stream) != cudaSuccess) {
    if (ev) cudaEventDestroy(ev);
    cudaGetLastError();
    cudaFree(p);
    return;
  }
  g_cache[{l.ctx, l.bytes}].push_back(Cached{p, ev});
  g_cached_bytes += l.bytes;
}

// On context destruction: cached blocks are freed, live ones lose their context.
void dev_forget_ctx(blqh_ctx* ctx) {
  std::lock_guard<std::mutex> lk(g_mem_mu);
  release_cached(ctx);
  for (auto& kv : g_live)
    if (kv.second.ctx == ctx) kv.second.ctx = nullptr;
}

cudaError_t smem_attr_at_least(const void* func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, int> cur;  // (device, kernel) -> limit set
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  int& c = cur[{dev, func}];
  if (bytes <= c) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) c = bytes;
  return e;
}

int grid_for(blqh_ctx* ctx, int64_t work_items, int block, int per_sm_cap) {
  int64_t need = (work_items + block - 1) / block;
  int64_t cap = (int64_t)ctx->num_sms * per_sm_cap;
  if (need > cap) need = cap;
  if (need < 1) need = 1;
  return (int)need;
}

// ---------------------------------------------------------------------------
TimerScope::TimerScope(blqh_ctx* c, int k) : ctx(c), cls(k) {
  if (!ctx->timing) return;
  if (ctx->ev_pool.size() < 2) {
    for (int i = 0; i < 64; i++) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ctx->ev_pool.push_back(e);
    }
  }
  a = ctx->ev_pool.back();
  ctx->ev_pool.pop_back();
  b = ctx->ev_pool.back();
  ctx->ev_pool.pop_back();
  cudaEventRecord(a, ctx->stream);
}

TimerScope::~TimerScope() {
  if (!a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->pending.push_back({cls, {a, b}});
  if (ctx->pending.size() > 512) flush_timers(ctx);
}

void count_launch(blqh_ctx* ctx, int cls, int n) { ctx->launches[cls] += n; }

void flush_timers(blqh_ctx* ctx) {
  if (ctx->pending.empty()) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, p.second.first, p.second.second);
    ctx->ms[p.first] += ms;
    ctx->ev_pool.push_back(p.second.first);
    ctx->ev_pool.push_back(p.second.second);
  }
  ctx->pending.clear();
}

// ---------------------------------------------------------------------------
// Exclusive scan: per-block sums, a single-block scan of the block sums, then
// a per-block scan with the block offset. Deterministic.
namespace {
constexpr int SCAN_BLOCK = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <class T>
__device__ int64_t block_sum_tile(const T* in, int64_t n, int64_t base) {
  int64_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; k++) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < n) s += (int64_t)in[i];
  }
  return s;
}

__device__ int64_t block_exclusive(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[SCAN_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t w = (lane < SCAN_BLOCK / 32) ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_BLOCK / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  int64_t off = (wid > 0) ? warp_sums[wid - 1] : 0;
  if (total) *total = warp_sums[SCAN_BLOCK / 32 - 1];
  int64_t r = off + x - v;
  __syncthreads();
  return r;
}

template <class T>
__global__ void k_scan_reduce(const T* in, int64_t n, int64_t* block_sums) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t s = block_sum_tile(in, n, base);
  int64_t tot;
  block_exclusive(s, &tot);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void k_scan_blocks(int64_t* block_sums, int64_t nb, int64_t* total) {
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += SCAN_BLOCK) {
    int64_t i = base + threadIdx.x;
    int64_t v = (i < nb) ? block_sums[i] : 0;
    int64_t tot;
    int64_t ex = block_exclusive(v, &tot);
    if (i < nb) block_sums[i] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

template <class T>
__global__ void k_scan_apply(const T* in, int64_t* out, int64_t n, const int64_t* block_offs) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t vals[SCAN_ITEMS];
  int64_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; k++) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    vals[k] = (i < n) ? (int64_t)in[i] : 0;
    s += vals[k];
  }
  int64_t ex = block_exclusive(s, nullptr) + block_offs[blockIdx.x];
  for (int k = 0; k < SCAN_ITEMS; k++) {
    int64_t i = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (i < n) out[i] = ex;
    ex += vals[k];
  }
}

template <class T>
void scan_impl(blqh_ctx* ctx, const T* in, int64_t* out, int64_t n, int64_t* total_host) {
  if (n <= 0) {
    if (total_host) *total_host = 0;
    return;
  }
  int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  int64_t* bs = dalloc<int64_t>(ctx, nb + 1);
  k_scan_reduce<T><<<(unsigned)nb, SCAN_BLOCK, 0, ctx->stream>>>(in, n, bs);
  k_scan_blocks<<<1, SCAN_BLOCK, 0, ctx->stream>>>(bs, nb, bs + nb);
  k_scan_apply<T><<<(unsigned)nb, SCAN_BLOCK, 0, ctx->stream>>>(in, out, n, bs);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_MISC, 3);
  if (total_host) {
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(total_host, bs + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dev_free(bs);
}
}  // namespace

void scan_exclusive_i64(blqh_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total_host) {
  scan_impl<int64_t>(ctx, in, out, n, total_host);
}
void scan_exclusive_u32_to_i64(blqh_ctx* ctx, const uint32_t* in, int64_t* out, int64_t n, int64_t* total_host) {
  scan_impl<uint32_t>(ctx, in, out, n, total_host);
}

// ---------------------------------------------------------------------------
extern "C" {

int blqh_ctx_create(int device, blqh_ctx** out) {
  if (!out) return BLQH_ERR_ARG;
  *out = nullptr;
  blqh_ctx* c = new blqh_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&c->pinned, 4096);
  if (e != cudaSuccess) {
    set_error(nullptr, BLQH_ERR_CUDA, std::string("blqh_ctx_create: ") + cudaGetErrorString(e));
    delete c;
    return BLQH_ERR_CUDA;
  }
  *out = c;
  return BLQH_OK;
}

int blqh_ctx_destroy(blqh_ctx* c) {
  if (!c) return BLQH_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  dev_forget_ctx(c);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.second.first);
    cudaEventDestroy(p.second.second);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  for (auto e : c->marks)
    if (e) cudaEventDestroy(e);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return BLQH_OK;
}

const char* blqh_last_error(const blqh_ctx* c) {
  if (c && !c->last_error.empty()) return c->last_error.c_str();
  return g_thread_error.c_str();
}

int blqh_ctx_synchronize(blqh_ctx* c) {
  if (!c) return BLQH_ERR_ARG;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    set_error(c, BLQH_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    return BLQH_ERR_CUDA;
  }
  return BLQH_OK;
}

int blqh_ctx_timers(blqh_ctx* c, int enable, double* ms_out4, int64_t* launches_out4) {
  if (!c) return BLQH_ERR_ARG;
  flush_timers(c);
  if (ms_out4)
    for (int i = 0; i < TM_N; i++) ms_out4[i] = c->ms[i];
  if (launches_out4)
    for (int i = 0; i < TM_N; i++) launches_out4[i] = c->launches[i];
  if (enable >= 0) c->timing = enable != 0;
  return BLQH_OK;
}

int blqh_ctx_mark(blqh_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 8) return BLQH_ERR_ARG;
  if (!c->marks[slot] && cudaEventCreate(&c->marks[slot]) != cudaSuccess) return BLQH_ERR_CUDA;
  cudaError_t e = cudaEventRecord(c->marks[slot], c->stream);
  if (e != cudaSuccess) {
    set_error(c, BLQH_ERR_CUDA, std::string("blqh_ctx_mark: ") + cudaGetErrorString(e));
    return BLQH_ERR_CUDA;
  }
  return BLQH_OK;
}

int blqh_ctx_elapsed_ms(blqh_ctx* c, int a, int b, double* ms) {
  if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !c->marks[a] || !c->marks[b]) return BLQH_ERR_ARG;
  float f = 0;
  cudaError_t e = cudaEventSynchronize(c->marks[b]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&f, c->marks[a], c->marks[b]);
  if (e != cudaSuccess) {
    set_error(c, BLQH_ERR_CUDA, std::string("blqh_ctx_elapsed_ms: ") + cudaGetErrorString(e));
    return BLQH_ERR_CUDA;
  }
  *ms = f;
  return BLQH_OK;
}

int blqh_ctx_reset_timers(blqh_ctx* c) {
  if (!c) return BLQH_ERR_ARG;
  flush_timers(c);
  for (int i = 0; i < TM_N; i++) {
    c->ms[i] = 0;
    c->launches[i] = 0;
  }
  return BLQH_OK;
}

}  // extern "C"
