// Serving many small sparse requests with continuous batching.
//
// Matrices are registered once and stay resident in HBM.  A request names
// a matrix and carries a host input and a host output buffer.  Admission is
// by HBM footprint: a request is admitted when a request slot is free and
// its input + output fit in the server's device pool; otherwise it waits in
// the host queue and is admitted as soon as completions free memory.
// Page-locked buffers are read and written by the device directly: such an
// output takes no pool memory and needs no copy back.
//
// Batched mode (the device-side request loop).  A persistent kernel runs on
// every SM.  For each group of admitted requests the host writes one stage
// record per request into a page-locked ring and launches one stage kernel,
// which copies page-locked inputs into the pool, writes the slot
// descriptors and the work items -- blocks of rows_per_item rows of one
// request -- into device rings, and, from its last block, bumps the
// `published` counter in mapped host memory.  The host never waits for
// these copies.  Each block of the
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
constexpr int SRV_MAX_TAKE = 8;  // work items one claim may take
// Completion ring: the device appends one record per finished request; at most
// SRV_MAX_SLOTS records are unconsumed (a slot completes again only after the
// host has taken its previous record and re-admitted it), so twice that never
// overwrites one the host has not read.
constexpr int SRV_DONE_CAP = 2 * SRV_MAX_SLOTS;

struct __align__(16) DevMatrix {
  const int32_t* ptr;
  const int32_t* idx;
  const float* val;
  int32_t nrows, ncols, base, nnz;
  int32_t lanes;  // SpMV lanes per row (a power of two <= 32), from the matrix's size class
  int32_t rpi;    // rows per work item of per-call launches, from the matrix's size class
};

// Size classes of registered matrices by mean stored entries per row:
// class 0 holds means below 1, class c >= 1 means in [2^(c-1), 2^c), the
// last class everything above.  Each class has its own serving shape.
constexpr int SRV_CLASSES = 10;
inline int size_class(int64_t nnz, int64_t nrows) {
  const double mean = nrows > 0 ? (double)nnz / (double)nrows : 0.0;
  int c = 0;
  while (c < SRV_CLASSES - 1 && mean >= (double)(int64_t(1) << c)) ++c;
  return c;
}

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
  // completion records, written in claim order by the device: bits 0-11 the
  // slot, 12-43 the low 32 bits of the request's sequence number, 44-63 the
  // ring lap + 1 (mod 2^20) of the position, so the host knows an entry is new
  volatile uint64_t done_ring[SRV_DONE_CAP];
};

struct SrvArgs {
  const DevMatrix* mats;
  const DevSlot* slots;
  const DevItem* items;
  HostShared* host;                 // device alias of the mapped block
  unsigned long long* next_item;    // device counter
  unsigned int* done_items;         // per slot
  unsigned int* exit_epoch;         // device word: the last launch told to exit
  unsigned long long* done_count;   // device counter: completion records written
  const unsigned int* epoch_word;   // device word: this launch's number (bumped before each launch)
  uint64_t idle_ns;
};

// The graph node before every launch of the device loop: a new launch number.
__global__ void serve_bump_epoch_k(unsigned int* epoch_word) { *epoch_word += 1u; }

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

// y[r] = sum_j A[r,j] x[j] over the G lanes of one row group (gl = lane in
// the group; a row of r < 0 contributes nothing but still takes part in the
// shuffles); returns y[r] in every lane of the group.  Lanes stride the
// row's entries by G and the partial sums fold by xor over the group: a
// fixed order for each G.
__device__ float srv_spmv_row(const DevMatrix& A, const float* __restrict__ x, int r, int gl, int G) {
  float acc = 0.f;
  if (r >= 0) {
    const int q0 = __ldg(A.ptr + r) - A.base, q1 = __ldg(A.ptr + r + 1) - A.base;
    for (int q = q0 + gl; q < q1; q += G)
      acc = __fmaf_rn(__ldg(A.val + q), __ldcg(x + (__ldg(A.idx + q) - A.base)), acc);
  }
  for (int m = G >> 1; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
  return acc;
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

constexpr int SRV_YCHUNK = 256;  // SpMV rows staged in shared memory per store pass

__device__ void srv_process(const SrvArgs& a, const DevSlot& s, const DevItem& it) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DevMatrix A = ldcg_struct(a.mats + s.matrix);
  if (s.op == FGB_REQ_SPMV) {
    // one value per row: staged so that the block stores whole lines (the
    // output may live in host memory, where scattered 4-byte stores are slow)
    __shared__ float s_y[SRV_YCHUNK];
    const int G = A.lanes, per = 32 / G, sub = lane / G, gl = lane % G;  // 32 / G rows per warp at once
    for (int r0 = (int)it.row_begin; r0 < (int)it.row_end; r0 += SRV_YCHUNK) {
      const int n = min(SRV_YCHUNK, (int)it.row_end - r0);
      for (int k0 = warp * per; k0 < n; k0 += (SRV_THREADS / 32) * per) {
        const int k = k0 + sub;
        const float y = srv_spmv_row(A, s.in, k < n ? r0 + k : -1, gl, G);
        if (k < n && gl == 0) s_y[k] = y;
      }
      __syncthreads();
      for (int k = threadIdx.x; k < n; k += SRV_THREADS) s.out[r0 + k] = s_y[k];
      __syncthreads();
    }
    return;
  }
  const DevMatrix Bm = s.op == FGB_REQ_MASKED_MUL ? ldcg_struct(a.mats + s.matrix_b) : A;
  for (int r = (int)it.row_begin + warp; r < (int)it.row_end; r += SRV_THREADS / 32) {
    if (s.op == FGB_REQ_SPMM) srv_spmm_row(A, s.in, s.out, s.nk, r, lane);
    else srv_masked_row(A, Bm, s.out, r, lane);
  }
}

// The device-side request loop.
// 5 blocks' worth of registers per SM at most: with the default 4 blocks per
// SM there is room left for the stage kernel to run beside the loop.
//
// Idle exit is collective: a block leaves only when the shared item counter
// has not moved for idle_ns (no block claimed anything), and the first block
// to see that raises exit_epoch to this launch's epoch so that every block
// leaves.  The host relaunches when it sees the kernel finished with work
// outstanding; a kernel never keeps running on a few blocks.
__global__ void __launch_bounds__(SRV_THREADS, 5) serve_loop_k(SrvArgs a) {
  const unsigned epoch = *(volatile const unsigned*)a.epoch_word;  // set by the node before this launch
  __shared__ unsigned long long s_item;
  __shared__ unsigned s_take;
  __shared__ int s_exit;
  uint64_t cached_pub = 0;
  uint64_t idle_since = globaltimer();
  unsigned long long last_cur = ~0ull;
  while (true) {
    if (threadIdx.x == 0) {
      int exit_now = 0;
      unsigned long long got = 0;
      unsigned take = 0;
      unsigned backoff = 64;
      unsigned long long cur = *(volatile unsigned long long*)a.next_item;
      while (true) {
        if (cur < cached_pub) {
          // guided claiming: a share of the backlog, so that a deep backlog
          // costs few compare-and-swaps on the shared counter
          const unsigned long long share = (cached_pub - cur) / (2ull * gridDim.x);
          const unsigned want = share < 1 ? 1u : (share > SRV_MAX_TAKE ? (unsigned)SRV_MAX_TAKE : (unsigned)share);
          const unsigned long long old = atomicCAS(a.next_item, cur, cur + want);
          if (old == cur) {
            got = cur;
            take = want;
            break;
          }
          cur = old;  // lost the race: retry from the counter's current value
          continue;
        }
        cached_pub = ld_acquire_sys(&a.host->published);
        if (cached_pub > cur) continue;
        if (a.host->stop || *(volatile unsigned*)a.exit_epoch >= epoch) { exit_now = 1; break; }
        const uint64_t now = globaltimer();
        if (cur != last_cur) {  // another block claimed an item: not idle
          last_cur = cur;
          idle_since = now;
        }
        if (now - idle_since > a.idle_ns) {
          atomicMax(a.exit_epoch, epoch);
          exit_now = 1;
          break;
        }
        __nanosleep(backoff);
        if (backoff < 4096) backoff <<= 1;
        cur = *(volatile unsigned long long*)a.next_item;
      }
      s_item = got;
      s_take = take;
      s_exit = exit_now;
    }
    __syncthreads();
    const int exit_now = s_exit;
    const unsigned long long first = s_item;
    const unsigned take = s_take;
    __syncthreads();
    if (exit_now) return;
    for (unsigned k = 0; k < take; ++k) {
      const DevItem it = ldcg_struct(a.items + (first + k) % SRV_ITEM_CAP);
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
          const unsigned long long pos = atomicAdd(a.done_count, 1ull);
          const uint64_t lap = ((uint64_t)(pos / SRV_DONE_CAP) + 1u) & 0xFFFFFull;
          const uint64_t rec = (lap << 44) | ((uint64_t)(uint32_t)s.seq << 12) | (uint64_t)it.slot;
          __threadfence_system();
          st_release_sys(&a.host->done_ring[pos % SRV_DONE_CAP], rec);
        }
      }
    }
    if (threadIdx.x == 0) idle_since = globaltimer();
  }
}

// One admitted request, written by the host into a page-locked ring and read
// by the stage kernel.
struct __align__(16) StageReq {
  DevSlot desc;
  const float* src;  // device alias of a page-locked input (null: none or copied by DMA)
  float* dst;        // the input's pool range
  uint64_t bytes;    // bytes the stage kernel copies from src to dst
  uint64_t item0;    // ring index of the request's first work item
  int32_t slot, rows;
  int32_t rows_per_item, pad;
};

constexpr int STAGE_CAP = 2 * SRV_MAX_SLOTS;
constexpr uint32_t STAGE_CHUNK = 32u << 10;  // input bytes per stage block
constexpr int STAGE_THREADS = 256;

struct StageArgs {
  const StageReq* reqs;  // device alias of the ring
  uint32_t first, cap;
  DevSlot* slots;
  DevItem* items;
  unsigned* blocks_done;  // device counter, 0 between launches
  HostShared* host;
  uint64_t publish_to;
};

// Grid (x: STAGE_CHUNK input chunks, y: requests of the group).  Block x == 0
// of each request also writes its slot descriptor and work items.  The last
// block to finish publishes the group's items to the device loop.
__global__ void __launch_bounds__(STAGE_THREADS, 8) serve_stage_k(StageArgs g) {
  const StageReq* rq = g.reqs + (g.first + blockIdx.y) % g.cap;
  if (blockIdx.x == 0) {
    const int slot = rq->slot;
    if (threadIdx.x < (int)(sizeof(DevSlot) / 16))
      __stcg(reinterpret_cast<uint4*>(g.slots + slot) + threadIdx.x,
             reinterpret_cast<const uint4*>(&rq->desc)[threadIdx.x]);
    const int rpi = rq->rows_per_item, rows = rq->rows;
    const uint64_t item0 = rq->item0;
    for (int b = threadIdx.x; b < rq->desc.n_items; b += blockDim.x) {
      const uint4 it = make_uint4((uint32_t)slot, (uint32_t)(b * rpi), (uint32_t)min(rows, (b + 1) * rpi), 0u);
      __stcg(reinterpret_cast<uint4*>(g.items + (item0 + b) % SRV_ITEM_CAP), it);
    }
  }
  const uint64_t bytes = rq->bytes, c0 = (uint64_t)blockIdx.x * STAGE_CHUNK;
  if (c0 < bytes) {
    const uint64_t len = bytes - c0 < STAGE_CHUNK ? bytes - c0 : STAGE_CHUNK;
    const char* src = reinterpret_cast<const char*>(rq->src) + c0;
    char* dst = reinterpret_cast<char*>(rq->dst) + c0;
    uint64_t done = 0;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
      const uint64_t n16 = len >> 4;
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      uint4* d4 = reinterpret_cast<uint4*>(dst);
      for (uint64_t k = threadIdx.x; k < n16; k += blockDim.x) __stcg(d4 + k, __ldg(s4 + k));
      done = n16 << 4;
    }
    const uint32_t* s1 = reinterpret_cast<const uint32_t*>(src + done);  // inputs are float arrays
    uint32_t* d1 = reinterpret_cast<uint32_t*>(dst + done);
    for (uint64_t k = threadIdx.x; k < (len - done) >> 2; k += blockDim.x) __stcg(d1 + k, __ldg(s1 + k));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned total = gridDim.x * gridDim.y;
    if (atomicAdd(g.blocks_done, 1u) == total - 1) {
      *g.blocks_done = 0u;  // re-armed for the next stage launch (same stream)
      __threadfence_system();
      st_release_sys(&g.host->published, g.publish_to);
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
  const float* in_mapped = nullptr;  // device alias of a pinned input: copied by the stage kernel
  std::chrono::steady_clock::time_point t_submit, t_admit, t_done;
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
  StageReq* stage = nullptr;       // page-locked ring of stage records (host view)
  StageReq* stage_dev = nullptr;   // device view
  uint64_t stage_head = 0;         // records written so far
  std::vector<uint64_t> stage_pub; // per ring position: the published count its group reaches
  cudaStream_t copy_stream = nullptr, kernel_stream = nullptr;
  cudaEvent_t kernel_done = nullptr;
  bool kernel_launched = false;
  // the device loop's launch (epoch bump + loop kernel) and the stage launch,
  // each captured once into a graph that the dispatcher replays; the stage
  // node's grid and arguments are updated per group before its replay
  cudaGraphExec_t loop_exec = nullptr, stage_exec = nullptr;
  cudaGraph_t loop_graph = nullptr, stage_graph = nullptr;
  cudaGraphNode_t stage_node = nullptr;
  // serving shape per size class: SpMV lanes per row and rows per work item
  int32_t class_lanes[SRV_CLASSES] = {};
  int32_t class_rpi[SRV_CLASSES] = {};
  // host bookkeeping
  std::vector<DevMatrix> mats;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Ticket> tickets;
  std::vector<uint64_t> slot_owner;  // ticket per slot (0 = free)
  std::vector<int> free_slots;       // stack of slots with slot_owner == 0
  std::vector<uint64_t> slot_seq;
  struct Inflight {
    uint64_t id, seq, item0;
    int slot;
  };
  // admitted requests in admission order (worker only); an entry is complete
  // once slot_done_seq[slot] has reached its seq, and leaves from the front
  std::deque<Inflight> inflight;
  size_t n_inflight = 0;             // admitted, not yet complete
  std::vector<uint64_t> slot_done_seq;
  uint64_t done_cursor = 0;          // completion records consumed
  std::vector<uint64_t> done_scratch;
  std::vector<uint64_t> done_recs;
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

// Rows per work item of a request on A: the class's tuned value for the
// per-call launches (where it sets the grid, so the latency), the configured
// one for the batched loop (where it sets how many items are staged and
// claimed).  Items only split rows; a row's sum is the same either way.
int item_rows(const fgb_server* s, const DevMatrix& A) {
  return s->cfg.mode == FGB_SERVE_PER_CALL ? A.rpi : s->cfg.rows_per_item;
}

SrvArgs make_args(fgb_server* s) {
  SrvArgs a;
  a.mats = s->d_mats;
  a.slots = s->d_slots;
  a.items = s->d_items;
  a.host = s->host_dev;
  a.next_item = s->d_next;
  a.done_items = s->d_done;
  a.exit_epoch = (unsigned*)(s->d_next + 2);
  a.done_count = s->d_next + 3;
  a.epoch_word = (const unsigned*)(s->d_next + 4);
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
  s->stats.queue_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t.t_admit - t.t_submit).count();
  s->stats.service_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(t.t_done - t.t_admit).count();
  if (t.slot >= 0) {
    s->slot_owner[t.slot] = 0;
    s->free_slots.push_back(t.slot);
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
                                                                           item_rows(s, s->mats[r.matrix]));
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
  using clk = std::chrono::steady_clock;
  auto ns_since = [](clk::time_point t0) {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now() - t0).count();
  };
  while (!s->quit.load()) {
    bool progressed = false;
    s->stats.iterations++;
    const auto t_admit = clk::now();
    // A) admission: FIFO while a slot and pool memory are available
    std::vector<uint64_t> admitted;
    // ring positions still owned by in-flight requests start at the oldest one
    while (!s->inflight.empty() && s->slot_done_seq[s->inflight.front().slot] >= s->inflight.front().seq)
      s->inflight.pop_front();  // complete: its items no longer hold the ring
    const uint64_t ring_tail = s->inflight.empty() ? s->published : s->inflight.front().item0;
    int64_t new_items = 0;
    while (!s->queue.empty() && s->worker_error == FGB_OK) {
      Ticket& t = s->tickets[s->queue.front()];
      if ((int64_t)(s->published - ring_tail) + new_items + t.n_items > SRV_ITEM_CAP) break;
      if (s->free_slots.empty()) break;
      // the stage record this request would overwrite must have been consumed
      if (s->stage_pub[(s->stage_head + admitted.size()) % STAGE_CAP] > s->host->published) break;
      const int slot = s->free_slots.back();
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
      t.t_admit = clk::now();
      t.item0 = s->published + new_items;
      new_items += t.n_items;
      s->free_slots.pop_back();
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
      // one stage record per request, then one stage kernel for the group;
      // pageable inputs go by DMA on the same stream first
      cudaError_t e = cudaSuccess;
      int64_t n_new = 0;
      const uint64_t first = s->stage_head % STAGE_CAP;
      uint64_t max_chunks = 1;
      for (uint64_t id : admitted) {
        Ticket& t = s->tickets[id];
        float* in_pool = (float*)(s->pool + t.in_off);
        if (t.in_bytes && !t.in_mapped && e == cudaSuccess)
          e = cudaMemcpyAsync(in_pool, t.req.input, t.in_bytes, cudaMemcpyHostToDevice, s->copy_stream);
        StageReq& rq = s->stage[s->stage_head % STAGE_CAP];
        rq.desc = DevSlot{t.req.op, t.req.matrix, t.req.matrix_b, t.req.nk, in_pool,
                          t.out_mapped ? t.out_mapped : (float*)(s->pool + t.out_off),
                          (int32_t)t.n_items, 0, t.seq};
        rq.src = t.in_mapped;
        rq.dst = in_pool;
        rq.bytes = t.in_mapped ? t.in_bytes : 0;
        rq.item0 = t.item0;
        rq.slot = t.slot;
        rq.rows = (int32_t)t.rows;
        rq.rows_per_item = item_rows(s, s->mats[t.req.matrix]);
        rq.pad = 0;
        max_chunks = std::max<uint64_t>(max_chunks, (rq.bytes + STAGE_CHUNK - 1) / STAGE_CHUNK);
        n_new += t.n_items;
        ++s->stage_head;
      }
      const uint64_t publish_to = s->published + n_new;
      for (uint64_t k = 0; k < admitted.size(); ++k) s->stage_pub[(first + k) % STAGE_CAP] = publish_to;
      if (e == cudaSuccess) {
        StageArgs g{s->stage_dev, (uint32_t)first, (uint32_t)STAGE_CAP, s->d_slots, s->d_items,
                    (unsigned*)(s->d_next + 1), s->host_dev, publish_to};
        // the captured stage launch, with this group's grid and arguments
        void* args[] = {&g};
        cudaKernelNodeParams kp{};
        kp.func = (void*)serve_stage_k;
        kp.gridDim = dim3((unsigned)max_chunks, (unsigned)admitted.size());
        kp.blockDim = dim3(STAGE_THREADS);
        kp.kernelParams = args;
        e = cudaGraphExecKernelNodeSetParams(s->stage_exec, s->stage_node, &kp);
        if (e == cudaSuccess) e = cudaGraphLaunch(s->stage_exec, s->copy_stream);
      }
      if (e != cudaSuccess) {
        fail_worker(s, FGB_ECUDA, "stage launch", e);
        for (uint64_t id : admitted) finish(s, s->tickets[id], FGB_ECUDA);
        s->cv_done.notify_all();
        continue;
      }
      s->published = publish_to;  // the stage kernel makes it visible to the device loop
      for (uint64_t id : admitted) {
        const Ticket& t = s->tickets[id];
        s->inflight.push_back({id, t.seq, t.item0, t.slot});
        ++s->n_inflight;
      }
      s->stats.batches_published++;
    }
    s->stats.admit_ns += ns_since(t_admit);
    // B) keep the device loop running while work is outstanding
    if (s->cfg.mode == FGB_SERVE_BATCHED && s->n_inflight > 0) {
      const bool running = s->kernel_launched && cudaEventQuery(s->kernel_done) == cudaErrorNotReady;
      if (!running) {
        cudaGetLastError();
        // the captured relaunch: a new launch number, then the loop kernel
        cudaError_t e = cudaGraphLaunch(s->loop_exec, s->kernel_stream);
        if (e == cudaSuccess) e = cudaEventRecord(s->kernel_done, s->kernel_stream);
        if (e != cudaSuccess) fail_worker(s, FGB_ECUDA, "serve_loop_k launch", e);
        s->kernel_launched = true;
        s->stats.launches++;
      }
    }
    // C) completions: new records of the completion ring are read without the
    // lock (the cursor belongs to this thread, and submitters and waiters
    // must not queue behind it); copies back and releases take it again
    if (s->n_inflight > 0) {
      lk.unlock();
      const auto t_scan = clk::now();
      std::vector<uint64_t>& recs = s->done_recs;
      recs.clear();
      while (true) {
        const uint64_t want = ((s->done_cursor / SRV_DONE_CAP) + 1u) & 0xFFFFFull;
        const uint64_t rec = s->host->done_ring[s->done_cursor % SRV_DONE_CAP];
        if ((rec >> 44) != want) break;
        recs.push_back(rec);
        ++s->done_cursor;
      }
      const uint64_t scan_ns = ns_since(t_scan);
      lk.lock();
      s->stats.scan_ns += scan_ns;
      std::vector<uint64_t>& done = s->done_scratch;
      done.clear();
      for (uint64_t rec : recs) {
        const int slot = (int)(rec & 0xFFFull);
        const uint64_t id = s->slot_owner[slot];
        if (!id) continue;
        const Ticket& t = s->tickets[id];
        if ((uint32_t)(rec >> 12) != (uint32_t)t.seq) continue;  // not this admission's record
        s->slot_done_seq[slot] = t.seq;
        done.push_back(id);
      }
      s->n_inflight -= done.size();
      if (!done.empty()) {
        const auto t_fin = clk::now();
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
        s->cv_done.notify_all();
        s->stats.finish_ns += ns_since(t_fin);
      }
    }
    if (!progressed) {
      if (s->queue.empty() && s->n_inflight == 0)
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
  {
    // leave one block's room per SM for the stage kernel
    int occ = 0;
    FGB_CUDA_TRY(cudaSetDevice(ctx->device));
    FGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_loop_k, SRV_THREADS, 0));
    cfg.blocks_per_sm = std::max(1, std::min(cfg.blocks_per_sm, occ - 1));
  }
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
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&s->stage, sizeof(StageReq) * STAGE_CAP, cudaHostAllocMapped | cudaHostAllocPortable);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&s->stage_dev, s->stage, 0);
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
  for (int k = cfg.max_inflight - 1; k >= 0; --k) s->free_slots.push_back(k);
  s->slot_seq.assign(cfg.max_inflight, 0);
  s->slot_done_seq.assign(cfg.max_inflight, 0);
  s->stage_pub.assign(STAGE_CAP, 0);
  for (int c = 0; c < SRV_CLASSES; ++c) {
    s->class_lanes[c] = 32;
    s->class_rpi[c] = cfg.rows_per_item;
  }
  // capture the two launches the dispatcher replays (nothing runs here)
  {
    const int grid = ctx->num_sms * cfg.blocks_per_sm;
    cudaError_t ge = cudaStreamBeginCapture(s->kernel_stream, cudaStreamCaptureModeThreadLocal);
    if (ge == cudaSuccess) {
      serve_bump_epoch_k<<<1, 1, 0, s->kernel_stream>>>((unsigned*)(s->d_next + 4));
      serve_loop_k<<<grid, SRV_THREADS, 0, s->kernel_stream>>>(make_args(s));
      ge = cudaStreamEndCapture(s->kernel_stream, &s->loop_graph);
    }
    if (ge == cudaSuccess) ge = cudaGraphInstantiate(&s->loop_exec, s->loop_graph, 0);
    if (ge == cudaSuccess) ge = cudaStreamBeginCapture(s->copy_stream, cudaStreamCaptureModeThreadLocal);
    if (ge == cudaSuccess) {
      StageArgs g0{s->stage_dev, 0u, (uint32_t)STAGE_CAP, s->d_slots, s->d_items, (unsigned*)(s->d_next + 1),
                   s->host_dev, 0ull};
      serve_stage_k<<<dim3(1, 1), STAGE_THREADS, 0, s->copy_stream>>>(g0);
      ge = cudaStreamEndCapture(s->copy_stream, &s->stage_graph);
    }
    size_t nn = 1;
    if (ge == cudaSuccess) ge = cudaGraphGetNodes(s->stage_graph, &s->stage_node, &nn);
    if (ge == cudaSuccess) ge = cudaGraphInstantiate(&s->stage_exec, s->stage_graph, 0);
    if (ge != cudaSuccess) {
      set_error(FGB_ECUDA, "fgb_server_create: graphs: %s", cudaGetErrorString(ge));
      cudaGetLastError();
      fgb_server_destroy(s);
      return FGB_ECUDA;
    }
  }
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
  const int c = size_class(A->nnz, A->nrows);
  DevMatrix m{(const int32_t*)A->ptr, (const int32_t*)A->idx, (const float*)A->val, (int32_t)A->nrows,
              (int32_t)A->ncols, A->index_base, (int32_t)A->nnz, s->class_lanes[c], s->class_rpi[c]};
  FGB_CUDA_TRY(cudaMemcpy(s->d_mats + s->mats.size(), &m, sizeof(m), cudaMemcpyHostToDevice));
  *id = (int32_t)s->mats.size();
  s->mats.push_back(m);
  return FGB_OK;
}

}  // extern "C"

// Device aliases of page-locked request buffers (null for pageable memory);
// looked up before the server lock is taken.
struct MappedBufs {
  const float* in = nullptr;
  float* out = nullptr;
};

static void* device_alias(const void* p) {
  cudaPointerAttributes attr{};
  if (p && cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeHost)
    return attr.devicePointer;
  cudaGetLastError();
  return nullptr;
}

static MappedBufs probe_mapped(const fgb_request* r) {
  MappedBufs m;
  m.out = (float*)device_alias(r->output);
  if (r->op != FGB_REQ_MASKED_MUL) m.in = (const float*)device_alias(r->input);
  return m;
}

// Validates and queues one request; the caller holds s->mu.
static int submit_locked(fgb_server* s, const fgb_request* r, const MappedBufs& mb, uint64_t* ticket) {
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
  t.n_items = (A.nrows + item_rows(s, A) - 1) / item_rows(s, A);
  t.in_bytes = req_in_bytes(s, *r);
  t.out_bytes = req_out_bytes(s, *r, A.nnz);
  // a page-locked output is written by the device in place (no copy back);
  // a page-locked input is copied into the pool by the stage kernel
  if (mb.out) {
    t.out_mapped = mb.out;
    t.out_bytes = 0;
  }
  if (t.in_bytes) t.in_mapped = mb.in;
  if (t.in_bytes + t.out_bytes + 512 > s->cfg.pool_bytes)
    return set_error(FGB_ENOMEM, "fgb_server_submit: request needs %zu bytes, pool holds %zu",
                     t.in_bytes + t.out_bytes, s->cfg.pool_bytes);
  t.t_submit = std::chrono::steady_clock::now();
  const uint64_t id = s->next_ticket++;
  s->tickets.emplace(id, t);
  s->queue.push_back(id);
  s->stats.submitted++;
  *ticket = id;
  return FGB_OK;
}

// Waits for one ticket; the caller holds `lk` on s->mu.
static int wait_locked(fgb_server* s, std::unique_lock<std::mutex>& lk, uint64_t ticket,
                       int32_t timeout_ms, double* latency_s) {
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

extern "C" {

int fgb_server_submit(fgb_server* s, const fgb_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return set_error(FGB_EINVAL, "fgb_server_submit: null argument");
  const MappedBufs mb = probe_mapped(r);
  std::lock_guard<std::mutex> lk(s->mu);
  const int rc = submit_locked(s, r, mb, ticket);
  if (rc == FGB_OK) s->cv_work.notify_one();
  return rc;
}

int fgb_server_submit_batch(fgb_server* s, const fgb_request* reqs, int32_t n, uint64_t* tickets,
                            int32_t* n_accepted) {
  if (!s || (n > 0 && (!reqs || !tickets)) || !n_accepted)
    return set_error(FGB_EINVAL, "fgb_server_submit_batch: null argument");
  std::vector<MappedBufs> mb((size_t)std::max(n, 0));
  for (int32_t k = 0; k < n; ++k) mb[k] = probe_mapped(reqs + k);
  std::lock_guard<std::mutex> lk(s->mu);
  int rc = FGB_OK;
  int32_t k = 0;
  for (; k < n; ++k)
    if ((rc = submit_locked(s, reqs + k, mb[k], tickets + k)) != FGB_OK) break;
  *n_accepted = k;
  if (k) s->cv_work.notify_one();
  return rc;
}

int fgb_server_wait(fgb_server* s, uint64_t ticket, int32_t timeout_ms, double* latency_s) {
  if (!s) return set_error(FGB_EINVAL, "fgb_server_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  return wait_locked(s, lk, ticket, timeout_ms, latency_s);
}

int fgb_server_wait_batch(fgb_server* s, const uint64_t* tickets, int32_t n, int32_t timeout_ms,
                          double* latencies_s) {
  if (!s || (n > 0 && !tickets)) return set_error(FGB_EINVAL, "fgb_server_wait_batch: null argument");
  std::unique_lock<std::mutex> lk(s->mu);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  for (int32_t k = 0; k < n; ++k) {
    const auto left = std::chrono::duration_cast<std::chrono::milliseconds>(deadline - std::chrono::steady_clock::now());
    const int rc = wait_locked(s, lk, tickets[k], (int32_t)std::max<int64_t>(0, left.count()),
                               latencies_s ? latencies_s + k : nullptr);
    if (rc) return rc;
  }
  return FGB_OK;
}

}  // extern "C"

// Applies per-class shapes to the table and every registered matrix; the
// caller holds s->mu and the server is idle.
static int apply_shapes(fgb_server* s, const int32_t* lanes, const int32_t* rpi) {
  for (int c = 0; c < SRV_CLASSES; ++c) {
    s->class_lanes[c] = lanes[c];
    s->class_rpi[c] = rpi[c];
  }
  for (size_t k = 0; k < s->mats.size(); ++k) {
    DevMatrix& m = s->mats[k];
    const int c = size_class(m.nnz, m.nrows);
    m.lanes = lanes[c];
    m.rpi = rpi[c];
  }
  if (!s->mats.empty())
    FGB_CUDA_TRY(cudaMemcpy(s->d_mats, s->mats.data(), sizeof(DevMatrix) * s->mats.size(), cudaMemcpyHostToDevice));
  return FGB_OK;
}

static bool server_idle(const fgb_server* s) { return s->queue.empty() && s->n_inflight == 0; }

// The device loop leaves by itself once it has been idle for idle_exit_us;
// waits (bounded: that time plus a second) until it has, so that nothing
// else runs on the SMs.  False if it is still running.
static bool wait_loop_exit(const fgb_server* s) {
  if (!s->kernel_launched) return true;
  const auto limit = std::chrono::steady_clock::now() + std::chrono::microseconds(s->cfg.idle_exit_us) +
                     std::chrono::seconds(1);
  while (cudaEventQuery(s->kernel_done) == cudaErrorNotReady) {
    if (std::chrono::steady_clock::now() > limit) return false;
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  cudaGetLastError();
  return true;
}

// Makes the server's device current for a call made on a host thread of the
// caller's, and restores the caller's on the way out.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int device) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != device) cudaSetDevice(device);
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

extern "C" {

int fgb_server_tune(fgb_server* s, int32_t reps, fgb_server_tuning* out) {
  if (!s || !out) return set_error(FGB_EINVAL, "fgb_server_tune: null argument");
  if (reps <= 0) reps = 3;
  std::lock_guard<std::mutex> lk(s->mu);
  if (!server_idle(s)) return set_error(FGB_EBUSY, "fgb_server_tune: requests are in flight");
  if (!wait_loop_exit(s)) return set_error(FGB_EBUSY, "fgb_server_tune: the device loop has not exited");
  DeviceScope dev(s->ctx->device);
  *out = fgb_server_tuning{};
  static const int kLanes[] = {2, 4, 8, 16, 32};
  static const int kRpi[] = {32, 64, 128, 256};
  constexpr int kSample = 8;
  int64_t max_rows = 1, max_cols = 1;
  for (const DevMatrix& m : s->mats) {
    max_rows = std::max<int64_t>(max_rows, m.nrows);
    max_cols = std::max<int64_t>(max_cols, m.ncols);
  }
  DevMatrix* tmp = nullptr;
  float *x = nullptr, *y = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc((void**)&tmp, sizeof(DevMatrix) * kSample);
  if (e == cudaSuccess) e = cudaMalloc((void**)&x, sizeof(float) * max_cols);
  if (e == cudaSuccess) e = cudaMalloc((void**)&y, sizeof(float) * max_rows);
  if (e == cudaSuccess) e = cudaMemset(x, 0, sizeof(float) * max_cols);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  int32_t lanes[SRV_CLASSES], rpi[SRV_CLASSES];
  for (int c = 0; c < SRV_CLASSES; ++c) {
    lanes[c] = s->class_lanes[c];
    rpi[c] = s->class_rpi[c];
  }
  for (int c = 0; c < SRV_CLASSES && e == cudaSuccess; ++c) {
    std::vector<DevMatrix> sample;
    int count = 0;
    for (const DevMatrix& m : s->mats)
      if (size_class(m.nnz, m.nrows) == c) {
        ++count;
        if ((int)sample.size() < kSample) sample.push_back(m);
      }
    fgb_server_class_shape& o = out->cls[c];
    o.matrices = count;
    o.ms = o.ms_default = -1.0;
    o.lanes = lanes[c];
    o.rows_per_item = rpi[c];
    if (sample.empty()) continue;
    // the class's sample as SpMV requests through the serving kernel, at one shape
    auto time_shape = [&](int G, int R, double* ms) -> cudaError_t {
      std::vector<DevMatrix> t = sample;
      for (DevMatrix& m : t) {
        m.lanes = G;
        m.rpi = R;
      }
      cudaError_t ce = cudaMemcpyAsync(tmp, t.data(), sizeof(DevMatrix) * t.size(), cudaMemcpyHostToDevice, st);
      SrvArgs a = make_args(s);
      a.mats = tmp;
      for (int rep = -1; rep < reps && ce == cudaSuccess; ++rep) {  // rep -1: warm-up
        if (rep == 0) ce = cudaEventRecord(e0, st);
        for (int k = 0; k < (int)t.size() && ce == cudaSuccess; ++k) {
          const DevSlot slot{FGB_REQ_SPMV, k, -1, 0, x, y, (int32_t)((t[k].nrows + R - 1) / R), 0, 0};
          if (slot.n_items > 0) serve_one_k<<<(unsigned)slot.n_items, SRV_THREADS, 0, st>>>(a, slot, t[k].nrows, R);
          ce = cudaGetLastError();
        }
      }
      if (ce == cudaSuccess) ce = cudaEventRecord(e1, st);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float f = 0.f;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&f, e0, e1);
      *ms = f / reps;
      return ce;
    };
    double best = -1.0;
    for (int G : kLanes) {
      for (int R : kRpi) {
        double ms = 0;
        if ((e = time_shape(G, R, &ms)) != cudaSuccess) break;
        if (best < 0 || ms < best) {
          best = ms;
          lanes[c] = G;
          rpi[c] = R;
        }
      }
      if (e != cudaSuccess) break;
    }
    if (e == cudaSuccess) e = time_shape(32, s->cfg.rows_per_item, &o.ms_default);
    o.ms = best;
    o.lanes = lanes[c];
    o.rows_per_item = rpi[c];
  }
  int rc = FGB_OK;
  if (e != cudaSuccess) rc = set_error(FGB_ECUDA, "fgb_server_tune: %s", cudaGetErrorString(e));
  if (rc == FGB_OK) rc = apply_shapes(s, lanes, rpi);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(tmp);
  cudaFree(x);
  cudaFree(y);
  return rc;
}

int fgb_server_set_tuning(fgb_server* s, const fgb_server_tuning* t) {
  if (!s || !t) return set_error(FGB_EINVAL, "fgb_server_set_tuning: null argument");
  int32_t lanes[SRV_CLASSES], rpi[SRV_CLASSES];
  for (int c = 0; c < SRV_CLASSES; ++c) {
    const int G = t->cls[c].lanes, R = t->cls[c].rows_per_item;
    if (G < 1 || G > 32 || (G & (G - 1)) || R < 1 || R > (1 << 16))
      return set_error(FGB_EINVAL, "fgb_server_set_tuning: class %d: lanes %d, rows per item %d", c, G, R);
    lanes[c] = G;
    rpi[c] = R;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (!server_idle(s)) return set_error(FGB_EBUSY, "fgb_server_set_tuning: requests are in flight");
  return apply_shapes(s, lanes, rpi);
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
  if (s->loop_exec) cudaGraphExecDestroy(s->loop_exec);
  if (s->stage_exec) cudaGraphExecDestroy(s->stage_exec);
  if (s->loop_graph) cudaGraphDestroy(s->loop_graph);
  if (s->stage_graph) cudaGraphDestroy(s->stage_graph);
  if (s->kernel_done) cudaEventDestroy(s->kernel_done);
  if (s->kernel_stream) cudaStreamDestroy(s->kernel_stream);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->stage) cudaFreeHost(s->stage);
  if (s->host) cudaFreeHost(s->host);
  if (s->pool) cudaFree(s->pool);
  if (s->dev_state) cudaFree(s->dev_state);
  delete s->alloc;
  delete s;
  return FGB_OK;
}

}  // extern "C"
