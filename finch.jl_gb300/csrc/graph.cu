// Graph-program kernels: the `choose` and `minby` reductions of Finch's BFS
// and Bellman-Ford examples (docs/examples/bfs.jl, shortest_paths.jl), over
// the semantics of src/util/special_functions.jl:
//   choose(z)(a, b) = isequal(a, z) ? b : a   (the first value that is not z)
//   minby(a, b)     = a[1] > b[1] ? b : a     (the pair with the smaller first
//                                              component, ties to the left)
//
// Finch runs both programs as a push over the columns j of the adjacency
// (`for j=_, i=_` over Dense(SparseList)), so each output i sees its
// contributions in ascending j.  These kernels pull over the rows of the
// transposed storage (row i lists the j with edges[i, j]), one thread per
// row walking its entries in storage order -- ascending j -- so every
// output is the same left fold as Finch's, bit for bit, without atomics.
#include "fgb_internal.cuh"
#include "semiring.cuh"

namespace fgb {

template <class PtrT, class ParT>
__global__ void bfs_pull_k(int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx, int base,
                           const uint8_t* __restrict__ frontier, const uint8_t* __restrict__ visited,
                           ParT* __restrict__ parent, int64_t fill, int64_t offset, uint8_t* __restrict__ next) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nrows; k += (int64_t)gridDim.x * blockDim.x) {
    uint8_t hit = 0;
    if (!visited[k]) {
      const int64_t b = ld_ptr(ptr, k) - base, e = ld_ptr(ptr, k + 1) - base;
      int64_t first = INT64_MAX;  // the smallest j: the first one the j-ascending loop meets
      for (int64_t p = b; p < e; ++p) {
        const int64_t j = (int64_t)idx[p] - base;
        if (frontier[j] && j < first) first = j;
      }
      if (first != INT64_MAX) {
        hit = 1;
        if ((int64_t)parent[k] == fill) parent[k] = (ParT)(first + offset);  // choose(fill)
      }
    }
    next[k] = hit;
  }
}

// visited[k] |= next[k]; count += next[k] (block partial sums, then one atomic per block).
__global__ void or_count_k(int64_t n, uint8_t* __restrict__ visited, const uint8_t* __restrict__ next,
                           unsigned long long* __restrict__ count) {
  __shared__ unsigned long long part[32];
  unsigned long long mine = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t f = next[k] ? 1 : 0;
    visited[k] = visited[k] | f;
    mine += f;
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = mine;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long v = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0ull;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atomicAdd(count, v);  // integer sum: exact in any order
  }
}

// dst[j] <<minby>>= src[j] where mask[j] (the first loop of one relaxation round).
template <class T>
__global__ void minby_map_k(int64_t n, const uint8_t* __restrict__ mask, const T* __restrict__ src_d,
                            const int64_t* __restrict__ src_p, T* __restrict__ dst_d, int64_t* __restrict__ dst_p) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    if (mask && !mask[j]) continue;
    if (dst_d[j] > src_d[j]) {  // minby(dst, src) = dst[1] > src[1] ? src : dst
      dst_d[j] = src_d[j];
      dst_p[j] = src_p[j];
    }
  }
}

// One relaxation round (the second loop): for every active j and stored
// edges[i, j], d = dist_prev[j] + edges[i, j]; (dist[i], par[i]) <<minby>>=
// (d, j + offset); active[i] |= d < dist_prev[i].
template <class T, class PtrT>
__global__ void minby_relax_k(int64_t nrows, const PtrT* __restrict__ ptr, const int* __restrict__ idx,
                              const T* __restrict__ w, int base, const T* __restrict__ dprev,
                              const uint8_t* __restrict__ aprev, T* __restrict__ dist, int64_t* __restrict__ par,
                              uint8_t* __restrict__ active, int64_t offset) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrows; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = ld_ptr(ptr, i) - base, e = ld_ptr(ptr, i + 1) - base;
    T cd = dist[i];
    int64_t cp = par[i];
    const T di = dprev[i];
    uint8_t act = 0;
    for (int64_t p = b; p < e; ++p) {
      const int64_t j = (int64_t)idx[p] - base;
      if (!aprev[j]) continue;
      const T d = Semi<SR_PT, T>::add(dprev[j], w[p]);  // Julia's +: wraps for integers
      if (cd > d) {  // minby((cd, cp), (d, j)) = cd > d ? (d, j) : (cd, cp)
        cd = d;
        cp = j + offset;
      }
      act |= (d < di) ? 1 : 0;
    }
    dist[i] = cd;
    par[i] = cp;
    active[i] = act;
  }
}

template <class PtrT>
static int bfs_typed(fgb_ctx* ctx, const fgb_sparse* A, const uint8_t* frontier, const uint8_t* visited,
                     void* parent, int parent_t, int64_t fill, int64_t offset, uint8_t* next, cudaStream_t s) {
  const int grid = grid_for(A->nrows, 256, ctx->num_sms);
  const PtrT* ptr = (const PtrT*)A->ptr;
  if (parent_t == FGB_I64)
    bfs_pull_k<PtrT, int64_t><<<grid, 256, 0, s>>>(A->nrows, ptr, (const int*)A->idx, A->index_base, frontier,
                                                   visited, (int64_t*)parent, fill, offset, next);
  else
    bfs_pull_k<PtrT, int32_t><<<grid, 256, 0, s>>>(A->nrows, ptr, (const int*)A->idx, A->index_base, frontier,
                                                   visited, (int32_t*)parent, fill, offset, next);
  return check_launch("bfs_pull_k");
}

template <class T, class PtrT>
static int relax_typed(fgb_ctx* ctx, const fgb_sparse* A, const void* dprev, const uint8_t* aprev, void* dist,
                       int64_t* par, uint8_t* active, int64_t offset, cudaStream_t s) {
  minby_relax_k<T, PtrT><<<grid_for(A->nrows, 256, ctx->num_sms), 256, 0, s>>>(
      A->nrows, (const PtrT*)A->ptr, (const int*)A->idx, (const T*)A->val, A->index_base, (const T*)dprev, aprev,
      (T*)dist, par, active, offset);
  return check_launch("minby_relax_k");
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_bfs_pull(fgb_ctx* ctx, const fgb_sparse* A, const uint8_t* frontier, const uint8_t* visited,
                            void* parent, int parent_t, int64_t choose_fill, int64_t index_offset, uint8_t* next,
                            void* stream) {
  FGB_REQUIRE(ctx && A, "fgb_bfs_pull: null argument");
  int rc = check_sparse(A, "fgb_bfs_pull: A", true);
  if (rc) return rc;
  FGB_REQUIRE(A->orient == FGB_CSR, "fgb_bfs_pull: A must be CSR (row k lists the j with edges[k, j])");
  FGB_REQUIRE(parent_t == FGB_I32 || parent_t == FGB_I64, "fgb_bfs_pull: parent must be I32 or I64");
  if (A->nrows == 0) return FGB_OK;
  FGB_REQUIRE(visited && parent && next && (frontier || A->ncols == 0), "fgb_bfs_pull: null vector");
  cudaStream_t s = pick_stream(ctx, stream);
  return A->ptr_t == FGB_I32
             ? bfs_typed<int32_t>(ctx, A, frontier, visited, parent, parent_t, choose_fill, index_offset, next, s)
             : bfs_typed<int64_t>(ctx, A, frontier, visited, parent, parent_t, choose_fill, index_offset, next, s);
}

extern "C" int fgb_or_count(fgb_ctx* ctx, int64_t n, uint8_t* visited, const uint8_t* next, int64_t* count,
                            void* stream) {
  FGB_REQUIRE(ctx && count, "fgb_or_count: null argument");
  FGB_REQUIRE(n >= 0, "fgb_or_count: negative length");
  if (n == 0) return FGB_OK;
  FGB_REQUIRE(visited && next, "fgb_or_count: null vector");
  cudaStream_t s = pick_stream(ctx, stream);
  or_count_k<<<grid_for(n, 256, ctx->num_sms), 256, 0, s>>>(n, visited, next, (unsigned long long*)count);
  return check_launch("or_count_k");
}

extern "C" int fgb_minby_map(fgb_ctx* ctx, int dtype, int64_t n, const uint8_t* mask, const void* src_dist,
                             const int64_t* src_parent, void* dst_dist, int64_t* dst_parent, void* stream) {
  FGB_REQUIRE(ctx, "fgb_minby_map: null ctx");
  FGB_REQUIRE(n >= 0, "fgb_minby_map: negative length");
  if (n == 0) return FGB_OK;
  FGB_REQUIRE(src_dist && src_parent && dst_dist && dst_parent, "fgb_minby_map: null vector");
  cudaStream_t s = pick_stream(ctx, stream);
  const int grid = grid_for(n, 256, ctx->num_sms);
  switch (dtype) {
    case FGB_F64:
      minby_map_k<double><<<grid, 256, 0, s>>>(n, mask, (const double*)src_dist, src_parent, (double*)dst_dist,
                                               dst_parent);
      break;
    case FGB_F32:
      minby_map_k<float><<<grid, 256, 0, s>>>(n, mask, (const float*)src_dist, src_parent, (float*)dst_dist,
                                              dst_parent);
      break;
    case FGB_I32:
      minby_map_k<int32_t><<<grid, 256, 0, s>>>(n, mask, (const int32_t*)src_dist, src_parent, (int32_t*)dst_dist,
                                                dst_parent);
      break;
    case FGB_I64:
      minby_map_k<int64_t><<<grid, 256, 0, s>>>(n, mask, (const int64_t*)src_dist, src_parent, (int64_t*)dst_dist,
                                                dst_parent);
      break;
    default: return set_error(FGB_EUNSUPPORTED, "fgb_minby_map: dtype %d", dtype);
  }
  return check_launch("minby_map_k");
}

extern "C" int fgb_minby_relax(fgb_ctx* ctx, const fgb_sparse* A, const void* dist_prev, const uint8_t* active_prev,
                               void* dist, int64_t* parent, uint8_t* active, int64_t index_offset, void* stream) {
  FGB_REQUIRE(ctx && A, "fgb_minby_relax: null argument");
  int rc = check_sparse(A, "fgb_minby_relax: A", true);
  if (rc) return rc;
  FGB_REQUIRE(A->orient == FGB_CSR, "fgb_minby_relax: A must be CSR (row i lists the j with edges[i, j])");
  FGB_REQUIRE(A->nrows == A->ncols, "fgb_minby_relax: the adjacency must be square");
  if (A->nrows == 0) return FGB_OK;
  FGB_REQUIRE(dist_prev && active_prev && dist && parent && active, "fgb_minby_relax: null vector");
  FGB_REQUIRE(dist_prev != dist, "fgb_minby_relax: dist_prev and dist must be different buffers");
  FGB_REQUIRE(A->nnz == 0 || A->val, "fgb_minby_relax: A needs edge weights");
  cudaStream_t s = pick_stream(ctx, stream);
  const bool i32 = A->ptr_t == FGB_I32;
  switch (A->val_t) {
    case FGB_F64:
      return i32 ? relax_typed<double, int32_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s)
                 : relax_typed<double, int64_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s);
    case FGB_F32:
      return i32 ? relax_typed<float, int32_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s)
                 : relax_typed<float, int64_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s);
    case FGB_I32:
      return i32 ? relax_typed<int32_t, int32_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s)
                 : relax_typed<int32_t, int64_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s);
    case FGB_I64:
      return i32 ? relax_typed<int64_t, int32_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s)
                 : relax_typed<int64_t, int64_t>(ctx, A, dist_prev, active_prev, dist, parent, active, index_offset, s);
    default: return set_error(FGB_EUNSUPPORTED, "fgb_minby_relax: weights of dtype %d", A->val_t);
  }
}
