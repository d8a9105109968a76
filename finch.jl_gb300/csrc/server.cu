// Serving many small sparse requests with continuous batching.
//
// Matrices are registered once and stay resident in HBM.  A request names
// a matrix and carries a host input and a host output buffer.  Admission is
// by HBM footprint: a request is admitted when a request slot is free and
// its input + output fit in the server's device pool; otherwise it waits in
// the host queue and is admitted as soon as completions free memory.
//
// Batched mode (the device-side request loop).  A persistent kernel runs on
// every SM.  The host publishes admitted requests as work items -- blocks of
// rows_per_item rows of one request -- into a ring in device memory and then
// bumps a `published` counter in mapped host memory.  Each block of the
// kernel claims the next published item with a compare-and-swap on a device
// counter, computes its rows (8 warps, one row per warp at a time), and the
// block finishing a request's last item raises that request's status in
// mapped memory.  Requests that arrive while others run are published into
// the same ring and picked up by the running kernel: their work overlaps on
// the device.  Every wait in the kernel is bounded: with no work for
// idle_exit_us it exits, and the host relaunches it when work arrives.
//
// Per-call mode (the plain GPU path it is compared against): the dispatcher
// runs one request at a time -- copy in, one kernel launch over that
// request's items, copy out, synchronise.
//
// Every row of every request is computed by one warp in a fixed order, so a
// request's result is bit-identical alone, in a batch, and in per-call mode.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fgb_internal.cuh"

namespace fgb {

constexpr int SRV_MAX_SLOTS = 4096;
constexpr int64_t SRV_ITEM_CAP = int64_t(1) << 20;
constexpr int SRV_MAX_MATRICES = 1 << 16;
constexpr int SRV_THREADS = 256;

struct __align__(16) DevMatrix {
  const int32_t* ptr;
  const int32_t* idx;
  const float* val;
  int32_t nrows, ncols, base, nnz;
};

struct __align__(16) DevSlot {
  int32_t op, matrix, matrix_b, nk;
  const float* in;
  float* out;
  int32_t n_items, pad;
  uint64_t seq;
};

struct __align__(16) DevItem {
  uint32_t slot, row_begin, row_end, pad;
};

// Descriptors are rewritten by the host (DMA) while the loop runs: read them
// through L2 only, never from a possibly stale L1 line.
template <class T>
__device__ __forceinline__ T ldcg_struct(const T* p) {
  static_assert(sizeof(T) % 16 == 0, "descriptor size");
  T v;
  const uint4* s = reinterpret_cast<const uint4*>(p);
  uint4* d = reinterpret_cast<uint4*>(&v);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 16); ++i) d[i] = __ldcg(s + i);
  return v;
}

struct HostShared {           // pinned, mapped into the device address space
  volatile uint64_t published;  // items published so far (host writes)
  volatile uint32_t stop;       // host asks the device loop to exit
  volatile uint32_t error;
  volatile uint64_t status[SRV_MAX_SLOTS];  // seq of the last completed request per slot
};

struct SrvArgs {
  const DevMatrix* mats;
  const DevSlot* slots;
  const DevItem* items;
  HostShared* host;                 // device alias of the mapped block
  unsigned long long* next_item;    // device counter
  unsigned int* done_items;         // per slot
  uint64_t idle_ns;
};

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint64_t ld_acquire_sys(const volatile uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_sys(volatile uint64_t* p, uint64_t v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// y[r] = sum_j A[r,j] x[j]
__device__ void srv_spmv_row(const DevMatrix& A, const float* __restrict__ x, float* __restrict__ y,
                             int r, int lane) {
  const int q0 = __ldg(A.ptr + r) - A.base, q1 = __ldg(A.ptr + r + 1) - A.base;
  float acc = 0.f;
  for (int q = q0 + lane; q < q1; q += 32)
    acc = __fmaf_rn(__ldg(A.val + q), __ldcg(x + (__ldg(A.idx + q) - A.base)), acc);
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
  if (lane == 0) y[r] = acc;
}

// C[r, 0:nk] = sum_j A[r,j] B[j, 0:nk]; nk a multiple of 4, at most 128.
__device__ void srv_spmm_row(const DevMatrix& A, const float* __restrict__ B, float* __restrict__ C,
                             int nk, int r, int lane) {
  const int L = nk >> 2;                 // lanes per entry
  const int P = L >= 32 ? 1 : 32 / L;    // entries in flight per warp (P * L <= 32)
  const int sub = lane / L, sl = lane % L;
  const bool active = sub < P;
  const int q0 = __ldg(A.ptr + r) - A.base, q1 = __ldg(A.ptr + r + 1) - A.base;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (active)
    for (int q = q0 + sub; q < q1; q += P) {
      const float a = __ldg(A.val + q);
      const float4 b = __ldcg(reinterpret_cast<const float4*>(B + (int64_t)(__ldg(A.idx + q) - A.base) * nk) + sl);
      acc.x = __fmaf_rn(a, b.x, acc.x);
      acc.y = __fmaf_rn(a, b.y, acc.y);
      acc.z = __fmaf_rn(a, b.z, acc.z);
      acc.w = __fmaf_rn(a, b.w, acc.w);
    }
  // fold the P sub-groups (lanes congruent mod L); fixed order
  for (int m = L; m < 32; m <<= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, m);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, m);
    acc.z += __shfl_xor_sync(0xffffffffu, acc.z, m);
    acc.w += __shfl_xor_sync(0xffffffffu, acc.w, m);
  }
  if (sub == 0) reinterpret_cast<float4*>(C + (int64_t)r * nk)[sl] = acc;
}

// out[q] = A.val[q] * B2[r, A.idx[q]] over A's stored entries of row r
// (0 where B2 stores nothing): the masked elementwise multiply on A's pattern.
__device__ void srv_masked_row(const DevMatrix& A, const DevMatrix& Bm, float* __restrict__ out,
                               int r, int lane) {
  const int q0 = __ldg(A.ptr + r) - A.base, q1 = __ldg(A.ptr + r + 1) - A.base;
  const int b0 = __ldg(Bm.ptr + r) - Bm.base, b1 = __ldg(Bm.ptr + r + 1) - Bm.base;
  for (int q = q0 + lane; q < q1; q += 32) {
    const int j = __ldg(A.idx + q) - A.base;
    int lo = b0, hi = b1;  // first position with idx >= j
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(Bm.idx + mid) - Bm.base < j) lo = mid + 1; else hi = mid;
    }
    const float bv = (lo < b1 && __ldg(Bm.idx + lo) - Bm.base == j) ? __ldg(Bm.val + lo) : 0.f;
    out[q] = __fmul_rn(__ldg(A.val + q), bv);  // ptr[0] - base == 0: positions are 0-based
  }
}

__device__ void srv_process(const SrvArgs& a, const DevSlot& s, const DevItem& it) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevMatrix A = ldcg_struct(a.mats + s.matrix);
  const DevMatrix Bm = s.op == FGB_REQ_MASKED_MUL ? ldcg_struct(a.mats + s.matrix_b) : A;
  for (int r = (int)it.row_begin + warp; r < (int)it.row_end; r += SRV_THREADS / 32) {
    if (s.op == FGB_REQ_SPMV) srv_spmv_row(A, s.in, s.out, r, lane);
    else if (s.op == FGB_REQ_SPMM) srv_spmm_row(A, s.in, s.out, s.nk, r, lane);
    else srv_masked_row(A, Bm, s.out, r, lane);
  }
}

// The device-side request loop.
__global__ void __launch_bounds__(SRV_THREADS) serve_loop_k(SrvArgs a) {
  __shared__ unsigned long long s_item;
  __shared__ int s_exit;
  uint64_t cached_pub = 0;
  uint64_t idle_since = globaltimer();
  while (true) {
    if (threadIdx.x == 0) {
      int exit_now = 0;
      unsigned long long got = ~0ull;
      unsigned backoff = 64;
      while (true) {
        const unsigned long long cur = *(volatile unsigned long long*)a.next_item;
        if (cur < cached_pub) {
          if (atomicCAS(a.next_item, cur, cur + 1) == cur) {
            got = cur;
            break;
          }
          continue;  // lost the race for item `cur`; try the next one
        }
        cached_pub = ld_acquire_sys(&a.host->published);
        if (cached_pub > cur) continue;
        if (a.host->stop) { exit_now = 1; break; }
        if (globaltimer() - idle_since > a.idle_ns) { exit_now = 1; break; }
        __nanosleep(backoff);
        if (backoff < 4096) backoff <<= 1;
      }
      s_item = got;
      s_exit = exit_now;
    }
    __syncthreads();
    const int exit_now = s_exit;
    const unsigned long long item = s_item;
    __syncthreads();
    if (exit_now) return;
    const DevItem it = ldcg_struct(a.items + item % SRV_ITEM_CAP);
    const DevSlot s = ldcg_struct(a.slots + it.slot);
    srv_process(a, s, it);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      const unsigned done = atomicAdd(a.done_items + it.slot, 1u) + 1u;
      if ((int)done == s.n_items) {
        // re-arm the slot's counter before the host can see the request done
        // (and hand the slot to the next request)
        a.done_items[it.slot] = 0u;
        __threadfence_system();
        st_release_sys(&a.host->status[it.slot], s.seq);
      }
      idle_since = globaltimer();
    }
  }
}

// Per-call mode: one launch computes one request (block b = item b).
__global__ void __launch_bounds__(SRV_THREADS) serve_one_k(SrvArgs a, DevSlot s, int rows, int rows_per_item) {
  DevItem it;
  it.slot = 0;
  it.row_begin = blockIdx.x * rows_per_item;
  it.row_end = min(rows, (int)(blockIdx.x + 1) * rows_per_item);
  srv_process(a, s, it);
}

// ---------------------------------------------------------------- host side

struct Ticket {
  fgb_request req{};
  int slot = -1;
  size_t in_off = 0, out_off = 0, in_bytes = 0, out_bytes = 0;
  int64_t rows = 0, n_items = 0;
  uint64_t item0 = 0;  // ring index of the request's first item
  uint64_t seq = 0;
  float* out_mapped = nullptr;  // device alias of a pinned output: written in place, no copy back
  std::chrono::steady_clock::time_point t_submit, t_done;
  int state = 0;  // 0 queued, 1 in flight, 2 done, 3 failed
  int status = FGB_OK;
};

struct PoolAllocator {  // first-fit over free ranges, 256-byte granules
  std::map<size_t, size_t> free_;
  size_t used = 0;
  explicit PoolAllocator(size_t bytes) { free_[0] = bytes; }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, start = it->first + bytes;
        free_.erase(it);
        if (rest) free_[start] = rest;
        used += bytes;
        return true;
      }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    used -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

}  // namespace fgb

using namespace fgb;

struct fgb_server {
  fgb_ctx* ctx = nullptr;
  fgb_server_config cfg{};
  // device state
  char* dev_state = nullptr;
  DevMatrix* d_mats = nullptr;
  DevSlot* d_slots = nullptr;
  DevItem* d_items = nullptr;
  unsigned long long* d_next = nullptr;
  unsigned int* d_done = nullptr;
  char* pool = nullptr;
  HostShared* host = nullptr;   // host view
  HostShared* host_dev = nullptr;  // device view
  DevItem* stage_items = nullptr;  // pinned staging
  DevSlot* stage_slots = nullptr;
  unsigned* zero_word = nullptr;   // pinned 0, copied to reset a slot's done counter
  cudaStream_t copy_stream = nullptr, kernel_stream = nullptr;
  cudaEvent_t kernel_done = nullptr;
  bool kernel_launched = false;
  // host bookkeeping
  std::vector<DevMatrix> mats;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Ticket> tickets;
  std::vector<uint64_t> slot_owner;  // ticket per slot (0 = free)
  std::vector<uint64_t> slot_seq;
  std::vector<uint64_t> inflight;
  uint64_t next_ticket = 1;
  uint64_t published = 0;
  PoolAllocator* alloc = nullptr;
  std::thread worker;
  std::atomic<bool> quit{false};
  fgb_server_stats stats{};
  int worker_error = FGB_OK;
  char worker_msg[256] = {0};
};

namespace {

size_t req_in_bytes(const fgb_server* s, const fgb_request& r) {
  const DevMatrix& A = s->mats[r.matrix];
  if (r.op == FGB_REQ_SPMV) return sizeof(float) * (size_t)A.ncols;
  if (r.op == FGB_REQ_SPMM) return sizeof(float) * (size_t)A.ncols * r.nk;
  return 0;
}

size_t req_out_bytes(const fgb_server* s, const fgb_request& r, int64_t nnz) {
  const DevMatrix& A = s->mats[r.matrix];
  if (r.op == FGB_REQ_SPMV) return sizeof(float) * (size_t)A.nrows;
  if (r.op == FGB_REQ_SPMM) return sizeof(float) * (size_t)A.nrows * r.nk;
  return sizeof(float) * (size_t)nnz;
}

SrvArgs make_args(fgb_server* s) {
  SrvArgs a;
  a.mats = s->d_mats;
  a.slots = s->d_slots;
  a.items = s->d_items;
  a.host = s->host_dev;
  a.next_item = s->d_next;
  a.done_items = s->d_done;
  a.idle_ns = (uint64_t)s->cfg.idle_exit_us * 1000ull;
  return a;
}

void fail_worker(fgb_server* s, int code, const char* what, cudaError_t e) {
  s->worker_error = code;
  snprintf(s->worker_msg, sizeof(s->worker_msg), "%s: %s", what, cudaGetErrorString(e));
}

void finish(fgb_server* s, Ticket& t, int status) {
  t.state = status == FGB_OK ? 2 : 3;
  t.status = status;
  t.t_done = std::chrono::steady_clock::now();
  if (t.slot >= 0) {
    s->slot_owner[t.slot] = 0;
    t.slot = -1;
  }
  if (t.in_bytes) s->alloc->release(t.in_off, t.in_bytes);
  if (t.out_bytes) s->alloc->release(t.out_off, t.out_bytes);
  t.in_bytes = t.out_bytes = 0;
  s->stats.completed++;
}

void run_per_call(fgb_server* s, std::vector<uint64_t>& batch, std::unique_lock<std::mutex>& lk) {
  for (uint64_t id : batch) {
    Ticket& t = s->tickets[id];
    const fgb_request r = t.req;
    float* out_dev = t.out_mapped ? t.out_mapped : (float*)(s->pool + t.out_off);
    const DevSlot slot{r.op, r.matrix, r.matrix_b, r.nk, (const float*)(s->pool + t.in_off),
                       out_dev, (int32_t)t.n_items, 0, t.seq};
    lk.unlock();
    cudaError_t e = cudaSuccess;
    if (t.in_bytes) e = cudaMemcpyAsync(s->pool + t.in_off, r.input, t.in_bytes, cudaMemcpyHostToDevice, s->copy_stream);
    if (e == cudaSuccess && t.n_items > 0) {
      serve_one_k<<<(unsigned)t.n_items, SRV_THREADS, 0, s->copy_stream>>>(make_args(s), slot, (int)t.rows,
                                                                           s->cfg.rows_per_item);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && !t.out_mapped)
      e = cudaMemcpyAsync(r.output, s->pool + t.out_off, t.out_bytes, cudaMemcpyDeviceToHost, s->copy_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_stream);
    lk.lock();
    s->stats.launches++;
    if (e != cudaSuccess) fail_worker(s, FGB_ECUDA, "per-call request", e);
    finish(s, t, e == cudaSuccess ? FGB_OK : FGB_ECUDA);
  }
  s->cv_done.notify_all();
}

void worker_main(fgb_server* s) {
  cudaSetDevice(s->ctx->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->quit.load()) {
    bool progressed = false;
    // A) admission: FIFO while a slot and pool memory are available
    std::vector<uint64_t> admitted;
    // ring positions still owned by in-flight requests start at the oldest one
    uint64_t ring_tail = s->published;
    for (uint64_t id : s->inflight) ring_tail = std::min(ring_tail, s->tickets[id].item0);
    int64_t new_items = 0;
    while (!s->queue.empty() && s->worker_error == FGB_OK) {
      Ticket& t = s->tickets[s->queue.front()];
      if ((int64_t)(s->published - ring_tail) + new_items + t.n_items > SRV_ITEM_CAP) break;
      int slot = -1;
      for (int k = 0; k < s->cfg.max_inflight; ++k)
        if (!s->slot_owner[k]) { slot = k; break; }
      if (slot < 0) break;
      size_t in_off = 0, out_off = 0;
      if (t.in_bytes && !s->alloc->alloc(t.in_bytes, &in_off)) break;
      if (t.out_bytes && !s->alloc->alloc(t.out_bytes, &out_off)) {
        if (t.in_bytes) s->alloc->release(in_off, t.in_bytes);
        break;
      }
      t.slot = slot;
      t.in_off = in_off;
      t.out_off = out_off;
      t.seq = ++s->slot_seq[slot];
      t.state = 1;
      t.item0 = s->published + new_items;
      new_items += t.n_items;
      s->slot_owner[slot] = s->queue.front();
      admitted.push_back(s->queue.front());
      s->queue.pop_front();
    }
    if (!admitted.empty()) {
      progressed = true;
      if (s->cfg.mode == FGB_SERVE_PER_CALL) {
        run_per_call(s, admitted, lk);
        continue;
      }
      // copy inputs, write slot descriptors and items, then publish
      cudaError_t e = cudaSuccess;
      int64_t n_new = 0;
      for (uint64_t id : admitted) {
        Ticket& t = s->tickets[id];
        if (t.in_bytes && e == cudaSuccess)
          e = cudaMemcpyAsync(s->pool + t.in_off, t.req.input, t.in_bytes, cudaMemcpyHostToDevice, s->copy_stream);
        s->stage_slots[t.slot] = DevSlot{t.req.op, t.req.matrix, t.req.matrix_b, t.req.nk,
                                        (const float*)(s->pool + t.in_off),
                                        t.out_mapped ? t.out_mapped : (float*)(s->pool + t.out_off),
                                        (int32_t)t.n_items, 0, t.seq};
        for (int64_t b = 0; b < t.n_items; ++b) {
          const int64_t pos = (s->published + n_new) % SRV_ITEM_CAP;
          s->stage_items[pos] = DevItem{(uint32_t)t.slot, (uint32_t)(b * s->cfg.rows_per_item),
                                        (uint32_t)std::min<int64_t>(t.rows, (b + 1) * s->cfg.rows_per_item), 0};
          ++n_new;
        }
      }
      // one copy of the slot table (in-flight slots are rewritten unchanged;
      // the device re-arms each slot's done counter itself)
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_slots, s->stage_slots, sizeof(DevSlot) * s->cfg.max_inflight,
                            cudaMemcpyHostToDevice, s->copy_stream);
      // the new items occupy ring positions [published, published + n_new)
      const int64_t p0 = s->published % SRV_ITEM_CAP;
      const int64_t first = std::min<int64_t>(n_new, SRV_ITEM_CAP - p0);
      if (e == cudaSuccess && first > 0)
        e = cudaMemcpyAsync(s->d_items + p0, s->stage_items + p0, sizeof(DevItem) * first, cudaMemcpyHostToDevice, s->copy_stream);
      if (e == cudaSuccess && n_new > first)
        e = cudaMemcpyAsync(s->d_items, s->stage_items, sizeof(DevItem) * (n_new - first), cudaMemcpyHostToDevice, s->copy_stream);
      lk.unlock();
      if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_stream);
      lk.lock();
      if (e != cudaSuccess) {
        fail_worker(s, FGB_ECUDA, "admission copies", e);
        for (uint64_t id : admitted) finish(s, s->tickets[id], FGB_ECUDA);
        s->cv_done.notify_all();
        continue;
      }
      s->published += n_new;
      std::atomic_thread_fence(std::memory_order_release);
      s->host->published = s->published;  // the device loop may now claim them
      for (uint64_t id : admitted) s->inflight.push_back(id);
      s->stats.batches_published++;
    }
    // B) keep the device loop running while work is outstanding
    if (s->cfg.mode == FGB_SERVE_BATCHED && !s->inflight.empty()) {
      const bool running = s->kernel_launched && cudaEventQuery(s->kernel_done) == cudaErrorNotReady;
      if (!running) {
        cudaGetLastError();
        const int grid = s->ctx->num_sms * s->cfg.blocks_per_sm;
        serve_loop_k<<<grid, SRV_THREADS, 0, s->kernel_stream>>>(make_args(s));
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(s->kernel_done, s->kernel_stream);
        if (e != cudaSuccess) fail_worker(s, FGB_ECUDA, "serve_loop_k launch", e);
        s->kernel_launched = true;
        s->stats.launches++;
      }
    }
    // C) completions: copy outputs back, free slots and pool memory
    if (!s->inflight.empty()) {
      std::vector<uint64_t> done, still;
      for (uint64_t id : s->inflight) {
        Ticket& t = s->tickets[id];
        if (s->host->status[t.slot] == t.seq) done.push_back(id); else still.push_back(id);
      }
      if (!done.empty()) {
        progressed = true;
        std::atomic_thread_fence(std::memory_order_acquire);
        cudaError_t e = cudaSuccess;
        bool copies = false;
        for (uint64_t id : done) {
          Ticket& t = s->tickets[id];
          if (e == cudaSuccess && !t.out_mapped) {
            e = cudaMemcpyAsync(t.req.output, s->pool + t.out_off, t.out_bytes, cudaMemcpyDeviceToHost, s->copy_stream);
            copies = true;
          }
        }
        if (copies) {
          lk.unlock();
          if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_stream);
          lk.lock();
        }
        if (e != cudaSuccess) fail_worker(s, FGB_ECUDA, "result copies", e);
        for (uint64_t id : done) finish(s, s->tickets[id], e == cudaSuccess ? FGB_OK : FGB_ECUDA);
        s->inflight.swap(still);
        s->cv_done.notify_all();
      }
    }
    if (!progressed) {
      if (s->queue.empty() && s->inflight.empty())
        s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
      else {
        lk.unlock();
        std::this_thread::yield();
        lk.lock();
      }
    }
  }
}

}  // namespace

extern "C" {

int fgb_server_create(fgb_ctx* ctx, const fgb_server_config* cfg_in, fgb_server** out) {
  if (!ctx || !out) return set_error(FGB_EINVAL, "fgb_server_create: null argument");
  *out = nullptr;
  fgb_server_config cfg = cfg_in ? *cfg_in : fgb_server_config{};
  if (cfg.pool_bytes == 0) cfg.pool_bytes = size_t(1) << 30;
  if (cfg.max_inflight <= 0) cfg.max_inflight = 1024;
  if (cfg.max_inflight > SRV_MAX_SLOTS) return set_error(FGB_EINVAL, "fgb_server_create: max_inflight above %d", SRV_MAX_SLOTS);
  if (cfg.rows_per_item <= 0) cfg.rows_per_item = 64;
  if (cfg.blocks_per_sm <= 0) cfg.blocks_per_sm = 4;
  if (cfg.idle_exit_us <= 0) cfg.idle_exit_us = 20000;
  if (cfg.mode != FGB_SERVE_BATCHED && cfg.mode != FGB_SERVE_PER_CALL)
    return set_error(FGB_EINVAL, "fgb_server_create: unknown mode");
  FGB_CUDA_TRY(cudaSetDevice(ctx->device));
  fgb_server* s = new fgb_server();
  s->ctx = ctx;
  s->cfg = cfg;
  const size_t st_bytes = sizeof(DevMatrix) * SRV_MAX_MATRICES + sizeof(DevSlot) * SRV_MAX_SLOTS +
                          sizeof(DevItem) * SRV_ITEM_CAP + 256 + sizeof(unsigned) * SRV_MAX_SLOTS;
  cudaError_t e = cudaMalloc((void**)&s->dev_state, st_bytes);
  if (e == cudaSuccess) e = cudaMemset(s->dev_state, 0, st_bytes);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->pool, cfg.pool_bytes);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->host, sizeof(HostShared), cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&s->host_dev, s->host, 0);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->stage_items, sizeof(DevItem) * SRV_ITEM_CAP, cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->stage_slots, sizeof(DevSlot) * SRV_MAX_SLOTS, cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->zero_word, 256, cudaHostAllocPortable);
  if (e == cudaSuccess) memset(s->zero_word, 0, 256);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->kernel_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->kernel_done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    int code = e == cudaErrorMemoryAllocation ? FGB_ENOMEM : FGB_ECUDA;
    set_error(code, "fgb_server_create: %s", cudaGetErrorString(e));
    cudaGetLastError();
    fgb_server_destroy(s);
    return code;
  }
  memset((void*)s->host, 0, sizeof(HostShared));
  char* p = s->dev_state;
  s->d_mats = (DevMatrix*)p;
  p += sizeof(DevMatrix) * SRV_MAX_MATRICES;
  s->d_slots = (DevSlot*)p;
  p += sizeof(DevSlot) * SRV_MAX_SLOTS;
  s->d_items = (DevItem*)p;
  p += sizeof(DevItem) * SRV_ITEM_CAP;
  s->d_next = (unsigned long long*)p;
  p += 256;
  s->d_done = (unsigned*)p;
  s->alloc = new PoolAllocator(cfg.pool_bytes);
  s->slot_owner.assign(cfg.max_inflight, 0);
  s->slot_seq.assign(cfg.max_inflight, 0);
  s->worker = std::thread(worker_main, s);
  *out = s;
  return FGB_OK;
}

int fgb_server_register(fgb_server* s, const fgb_sparse* A, int32_t* id) {
  if (!s || !id) return set_error(FGB_EINVAL, "fgb_server_register: null argument");
  int rc = check_sparse(A, "fgb_server_register: A", true);
  if (rc) return rc;
  if (A->orient != FGB_CSR || A->ptr_t != FGB_I32 || A->val_t != FGB_F32)
    return set_error(FGB_EUNSUPPORTED, "fgb_server_register: needs CSR with int32 ptr and F32 values");
  if (A->nrows > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "fgb_server_register: too many rows");
  std::lock_guard<std::mutex> lk(s->mu);
  if ((int)s->mats.size() >= SRV_MAX_MATRICES) return set_error(FGB_ENOMEM, "fgb_server_register: matrix table full");
  if (A->nnz > INT32_MAX) return set_error(FGB_EUNSUPPORTED, "fgb_server_register: too many entries");
  DevMatrix m{(const int32_t*)A->ptr, (const int32_t*)A->idx, (const float*)A->val, (int32_t)A->nrows,
              (int32_t)A->ncols, A->index_base, (int32_t)A->nnz};
  FGB_CUDA_TRY(cudaMemcpy(s->d_mats + s->mats.size(), &m, sizeof(m), cudaMemcpyHostToDevice));
  *id = (int32_t)s->mats.size();
  s->mats.push_back(m);
  return FGB_OK;
}

int fgb_server_submit(fgb_server* s, const fgb_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return set_error(FGB_EINVAL, "fgb_server_submit: null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->worker_error) return set_error(s->worker_error, "fgb_server_submit: server failed: %s", s->worker_msg);
  if (r->matrix < 0 || r->matrix >= (int)s->mats.size())
    return set_error(FGB_EINVAL, "fgb_server_submit: unknown matrix %d", r->matrix);
  const DevMatrix& A = s->mats[r->matrix];
  // SpMM rows are split into nk/4 lanes per entry: nk/4 must be a power of two
  if (r->op == FGB_REQ_SPMM && (r->nk < 4 || r->nk > 128 || (r->nk & 3) || ((r->nk >> 2) & ((r->nk >> 2) - 1))))
    return set_error(FGB_EUNSUPPORTED, "fgb_server_submit: SpMM width must be 4, 8, 16, 32, 64 or 128");
  if (r->op == FGB_REQ_MASKED_MUL) {
    if (r->matrix_b < 0 || r->matrix_b >= (int)s->mats.size())
      return set_error(FGB_EINVAL, "fgb_server_submit: unknown matrix_b %d", r->matrix_b);
    const DevMatrix& B = s->mats[r->matrix_b];
    if (B.nrows != A.nrows || B.ncols != A.ncols)
      return set_error(FGB_EINVAL, "fgb_server_submit: masked multiply of different shapes");
  } else if (r->op != FGB_REQ_SPMV && r->op != FGB_REQ_SPMM) {
    return set_error(FGB_EINVAL, "fgb_server_submit: unknown op %d", r->op);
  }
  if (!r->output || (r->op != FGB_REQ_MASKED_MUL && !r->input))
    return set_error(FGB_EINVAL, "fgb_server_submit: null input or output");
  Ticket t;
  t.req = *r;
  t.rows = A.nrows;
  t.n_items = (A.nrows + s->cfg.rows_per_item - 1) / s->cfg.rows_per_item;
  t.in_bytes = req_in_bytes(s, *r);
  t.out_bytes = req_out_bytes(s, *r, A.nnz);
  // a page-locked output is written by the device in place (no copy back)
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, r->output) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
      attr.devicePointer) {
    t.out_mapped = (float*)attr.devicePointer;
    t.out_bytes = 0;
  } else {
    cudaGetLastError();
  }
  if (t.in_bytes + t.out_bytes + 512 > s->cfg.pool_bytes)
    return set_error(FGB_ENOMEM, "fgb_server_submit: request needs %zu bytes, pool holds %zu",
                     t.in_bytes + t.out_bytes, s->cfg.pool_bytes);
  t.t_submit = std::chrono::steady_clock::now();
  const uint64_t id = s->next_ticket++;
  s->tickets.emplace(id, t);
  s->queue.push_back(id);
  s->stats.submitted++;
  *ticket = id;
  s->cv_work.notify_one();
  return FGB_OK;
}

int fgb_server_wait(fgb_server* s, uint64_t ticket, int32_t timeout_ms, double* latency_s) {
  if (!s) return set_error(FGB_EINVAL, "fgb_server_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return set_error(FGB_EINVAL, "fgb_server_wait: unknown ticket %llu", (unsigned long long)ticket);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  while (it->second.state < 2) {
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && it->second.state < 2)
      return set_error(FGB_ETIMEOUT, "fgb_server_wait: ticket %llu not done after %d ms",
                       (unsigned long long)ticket, timeout_ms);
  }
  const Ticket t = it->second;
  s->tickets.erase(it);
  if (latency_s) *latency_s = std::chrono::duration<double>(t.t_done - t.t_submit).count();
  if (t.status != FGB_OK) return set_error(t.status, "fgb_server_wait: request failed: %s", s->worker_msg);
  return FGB_OK;
}

int fgb_server_stats_get(fgb_server* s, fgb_server_stats* out) {
  if (!s || !out) return set_error(FGB_EINVAL, "fgb_server_stats_get: null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->pool_used = s->alloc ? s->alloc->used : 0;
  return FGB_OK;
}

int fgb_server_destroy(fgb_server* s) {
  if (!s) return FGB_OK;
  if (s->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->quit = true;
      s->cv_work.notify_all();
    }
    s->worker.join();
  }
  if (s->host) s->host->stop = 1;
  if (s->kernel_stream) cudaStreamSynchronize(s->kernel_stream);  // the loop exits on stop
  if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
  if (s->kernel_done) cudaEventDestroy(s->kernel_done);
  if (s->kernel_stream) cudaStreamDestroy(s->kernel_stream);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->stage_items) cudaFreeHost(s->stage_items);
  if (s->stage_slots) cudaFreeHost(s->stage_slots);
  if (s->zero_word) cudaFreeHost(s->zero_word);
  if (s->host) cudaFreeHost(s->host);
  if (s->pool) cudaFree(s->pool);
  if (s->dev_state) cudaFree(s->dev_state);
  delete s->alloc;
  delete s;
  return FGB_OK;
}

}  // extern "C"
