// Plans: an autotuned schedule for one operation on fixed operands, captured
// once into a CUDA graph and replayed.
//
// fgb_plan_create times each schedule of the operation's search space on the
// caller's own operands (lanes per fiber for SpMV; lanes per row group and
// merge-path item length for SpMM; lanes per entry and entry-chunk length
// for SDDMM), keeps the fastest, computes what depends only on the matrix
// (the SpMM merge-path item boundaries) and captures the launches of that
// schedule into a graph.  Choices are cached per shape class in the process
// (and in the file named by FGB_TUNE_CACHE, if set), so later plans for
// similar operands skip the search.  The graph binds the operand pointers
// given at creation: execute it after refreshing those buffers in place.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "fgb_internal.cuh"
#include "spmm_common.cuh"

namespace fgb {
int spmv_with_group(fgb_ctx* ctx, int semiring, const fgb_sparse* A, const void* x, int x_t,
                    void* y, int y_t, unsigned flags, int group, void* stream);
int sddmm_impl(fgb_ctx* ctx, const fgb_sparse* A, const void* X, int64_t ldx, const void* Y,
               int64_t ldy, int64_t k, void* out_val, int dtype, unsigned flags, int lanes,
               int64_t chunk, void* stream, int64_t slab);

struct Choice {
  int lanes = 0;
  int64_t path = 0;
  int panels = 1;  // SpMM: column panels (1 = the plain merge-path schedule)
  int variant = 0;  // SpMM: 0 register gathers, 1 TMA stage ring, 2 virtual-row slabs
  int bands = 1;    // virtual rows: column bands of A (1 = none)
};

static bool same_choice(const Choice& a, const Choice& b) {
  return a.lanes == b.lanes && a.path == b.path && a.panels == b.panels && a.variant == b.variant &&
         a.bands == b.bands;
}

static std::mutex g_tune_mu;
static std::map<std::string, Choice> g_tune_cache;
static bool g_tune_loaded = false;

static int bucket(int64_t v) { return v <= 0 ? 0 : (int)std::floor(std::log2((double)v) * 2.0); }

static std::string tune_key(const fgb_plan_desc* d) {
  const fgb_sparse* A = d->A;
  std::ostringstream k;
  k << d->op << ':' << d->semiring << ':' << d->dtype << ':' << (d->flags & FGB_FINCH_ORDER) << ':'
    << A->orient << ':' << A->val_t << ':' << bucket(A->nrows) << ':' << bucket(A->ncols) << ':'
    << bucket(A->nnz) << ':' << d->k;
  return k.str();
}

static void tune_cache_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("FGB_TUNE_CACHE");
  if (!path) return;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {  // key lanes path panels variant [bands]
    std::istringstream ls(line);
    std::string key;
    Choice c;
    if (!(ls >> key >> c.lanes >> c.path >> c.panels >> c.variant)) continue;
    if (!(ls >> c.bands)) c.bands = 1;
    g_tune_cache[key] = c;
  }
}

static void tune_cache_store_locked(const std::string& key, const Choice& c) {
  g_tune_cache[key] = c;
  const char* path = std::getenv("FGB_TUNE_CACHE");
  if (!path) return;
  std::ofstream out(path, std::ios::app);
  out << key << ' ' << c.lanes << ' ' << c.path << ' ' << c.panels << ' ' << c.variant << ' ' << c.bands
      << '\n';
}

// FGB_TUNE_LOG names a file that receives one line per timed candidate
// (shape key, lanes, path, panels, variant, bands, ms per run): the whole
// search, not only the choice.
static void tune_log(const std::string& key, const Choice& c, double ms) {
  const char* path = std::getenv("FGB_TUNE_LOG");
  if (!path) return;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::ofstream out(path, std::ios::app);
  out << key << ' ' << c.lanes << ' ' << c.path << ' ' << c.panels << ' ' << c.variant << ' ' << c.bands << ' '
      << ms << '\n';
}

}  // namespace fgb

using namespace fgb;

struct fgb_plan {
  std::map<int, fgb_panels*> panels;  // SpMM column-panel layouts by panel count
  std::map<std::pair<int64_t, int>, VrowSchedule> vrows;  // virtual-row schedules by (length, bands)
  void* partial = nullptr;            // their partial sums (largest candidate)
  size_t partial_bytes = 0;
  fgb_ctx* ctx = nullptr;
  fgb_plan_desc d{};
  fgb_sparse A{};
  Choice choice;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  fgb_plan_info info{};
};

namespace {

// Issues the operation with schedule `c` on stream s (no allocation, no sync).
int issue(fgb_plan* p, const Choice& c, cudaStream_t s, bool plan_ready) {
  const fgb_plan_desc& d = p->d;
  switch (d.op) {
    case FGB_PLAN_SPMV:
      return spmv_with_group(p->ctx, d.semiring, &p->A, d.in0, d.dtype, d.out, d.dtype, d.flags,
                             c.lanes, s);
    case FGB_PLAN_SPMM:
      if (c.panels > 1) {
        auto it = p->panels.find(c.panels);
        if (it == p->panels.end()) {
          fgb_panels* pn = nullptr;
          const int rc = fgb_panels_create(p->ctx, &p->A, c.panels, &pn);
          if (rc) return rc;
          it = p->panels.emplace(c.panels, pn).first;
        }
        fgb_spmm_tuning t{c.lanes, c.variant, c.path};
        return fgb_panels_spmm(p->ctx, it->second, d.in0, d.ld_in0, d.k, d.out, d.ld_out, d.dtype,
                               d.flags, &t, s);
      }
      if (c.variant == 2 || c.variant == 3) {
        auto it = p->vrows.find({c.path, c.bands});
        if (it == p->vrows.end()) {  // built outside capture (the timing pass comes first)
          VrowSchedule v;
          int rc = vrow_build(p->ctx, &p->A, (int)c.path, &v, s, false, c.bands);
          if (rc) return rc;
          it = p->vrows.emplace(std::make_pair(c.path, c.bands), v).first;
        }
        const size_t need = spmm_vrow_scratch_bytes(it->second, d.k);
        if (need > p->partial_bytes) {  // never during capture: the same choice ran before it
          cudaStreamSynchronize(s);
          cudaFree(p->partial);
          p->partial = nullptr;
          p->partial_bytes = 0;
          if (cudaMalloc(&p->partial, need) != cudaSuccess)
            return set_error(FGB_ENOMEM, "fgb_plan: partial sums (%zu bytes)", need);
          p->partial_bytes = need;
        }
        return spmm_vrow(p->ctx, it->second, &p->A, d.in0, d.ld_in0, d.k, d.out, d.ld_out,
                         (d.flags & FGB_ACCUMULATE) ? 1 : 0, 4 * c.lanes, p->partial, s, c.variant == 3);
      }
      if (c.path > 0)
        return spmm_merge(p->ctx, &p->A, d.in0, d.ld_in0, d.k, d.out, d.ld_out, d.dtype,
                          (d.flags & FGB_ACCUMULATE) ? 1 : 0, c.lanes, c.path, p->scratch,
                          p->scratch_bytes, s, plan_ready, nullptr, c.variant);
      return spmm_impl(p->ctx, &p->A, d.in0, d.ld_in0, d.k, d.out, d.ld_out, d.dtype, d.flags,
                       c.lanes, 0, s);
    case FGB_PLAN_SDDMM:
      if (c.variant == 3 || c.variant == 4) {  // virtual rows (schedule built outside capture); 4: cp.async gathers
        auto it = p->vrows.find({c.path, c.bands});
        if (it == p->vrows.end()) {
          VrowSchedule v;
          int rc = vrow_build(p->ctx, &p->A, (int)c.path, &v, s, false, c.bands);
          if (rc) return rc;
          it = p->vrows.emplace(std::make_pair(c.path, c.bands), v).first;
        }
        return sddmm_vrow(p->ctx, it->second, &p->A, d.in0, d.ld_in0, d.in1, d.ld_in1, d.k, d.out, s,
                          c.lanes > 0 ? 4 * c.lanes : 0, c.variant == 4);
      }
      return sddmm_impl(p->ctx, &p->A, d.in0, d.ld_in0, d.in1, d.ld_in1, d.k, d.out, d.dtype,
                        d.flags, c.lanes, c.path, s,
                        c.variant == 2 ? 128 / (d.dtype == FGB_F64 ? 8 : 4) : 0);
    default: return set_error(FGB_EINVAL, "fgb_plan: unknown op %d", d.op);
  }
}

std::vector<Choice> candidates(const fgb_plan* p) {
  std::vector<Choice> out;
  const fgb_plan_desc& d = p->d;
  if (d.op == FGB_PLAN_SPMV) {
    if (d.flags & FGB_FINCH_ORDER) return {Choice{1, 0}};
    for (int g : {1, 4, 8, 32}) out.push_back(Choice{g, 0});
    if (d.semiring != FGB_OR_AND && p->A.orient == FGB_CSR)
      out.push_back(Choice{2, 0});  // the adaptive pull: one lane per short row, a warp per long one
    if (d.semiring == FGB_OR_AND && p->A.orient == FGB_CSC)
      out.push_back(Choice{0, 0});  // the warp-cooperative push over the true columns
  } else if (d.op == FGB_PLAN_SPMM) {
    const int vn = d.dtype == FGB_F64 ? 2 : 4;
    const bool merge = p->A.orient == FGB_CSR && !(d.flags & FGB_FINCH_ORDER) && d.k % vn == 0 &&
                       d.ld_in0 % vn == 0 && d.ld_out % vn == 0 &&
                       (uintptr_t)d.in0 % (vn * (d.dtype == FGB_F64 ? 8 : 4)) == 0 &&
                       (uintptr_t)d.out % (vn * (d.dtype == FGB_F64 ? 8 : 4)) == 0;
    if (!merge) {
      for (int l : {4, 8, 16, 32}) out.push_back(Choice{l, 0});
      return out;
    }
    for (int l : {8, 16, 32})
      for (int64_t path : {128, 256, 512, 1024}) out.push_back(Choice{l, path, 1, 0});
    if (d.dtype == FGB_F32)  // B rows staged by TMA into a shared-memory ring
      for (int64_t path : {256, 512, 1024, 2048}) out.push_back(Choice{32, path, 1, 1});
    if (d.dtype == FGB_F32 && p->A.val_t == FGB_F32 && p->A.nrows <= INT32_MAX)
      for (int l : {2, 4, 8})  // column slabs over length-sorted virtual rows
        for (int64_t t : {32, 64, 128})
          for (int v : {2, 3}) out.push_back(Choice{l, t, 1, v});  // register / cp.async gathers
    // the same with A's columns cut into bands, so each launch gathers from
    // 1/bands of B's slab (worth it when the slab does not fit L2)
    if (d.dtype == FGB_F32 && p->A.val_t == FGB_F32 && p->A.nrows <= INT32_MAX && p->A.idx_t == FGB_I32 &&
        (double)p->A.ncols * 128.0 > 48.0 * 1024 * 1024)
      for (int l : {4, 8})
        for (int64_t t : {64, 128, 256})
          for (int nb : {2, 4, 8}) out.push_back(Choice{l, t, 1, 3, nb});
    // column panels keep each panel's slice of B in L2 (worth it when B is not)
    const double b_bytes = (double)p->A.ncols * (double)d.k * (d.dtype == FGB_F64 ? 8 : 4);
    if (b_bytes > 32.0 * 1024 * 1024 && !(d.flags & FGB_ACCUMULATE))
      for (int np : {4, 8, 16})
        for (int64_t path : {256, 512, 1024})
          for (int v : {0, 1})
            if (v == 0 || d.dtype == FGB_F32) out.push_back(Choice{32, path, np, v});
  } else {
    if (d.flags & FGB_FINCH_ORDER) return {Choice{0, 0}};
    for (int l : {4, 8, 16, 32})
      for (int64_t chunk : {128, 256, 512}) out.push_back(Choice{l, chunk});
    if (d.k * (d.dtype == FGB_F64 ? 8 : 4) > 128)  // column slabs of one 128-byte line
      for (int64_t chunk : {128, 256, 512}) out.push_back(Choice{d.dtype == FGB_F64 ? 16 : 8, chunk, 1, 2});
    if (d.dtype == FGB_F32 && p->A.orient == FGB_CSR && p->A.val_t == FGB_F32 && d.k <= 128 &&
        d.k % 4 == 0 && d.ld_in0 % 4 == 0 && d.ld_in1 % 4 == 0 && p->A.nnz <= INT32_MAX)
      for (int64_t t : {64, 128, 256}) {  // virtual rows, all of k or 32-column slabs
        for (int v : {3, 4}) {            // register / cp.async gathers
          out.push_back(Choice{0, t, 1, v});
          if (d.k > 32) out.push_back(Choice{8, t, 1, v});
        }
        if ((double)p->A.ncols * 128.0 > 48.0 * 1024 * 1024)  // column bands of A
          for (int nb : {2, 4, 8}) {
            out.push_back(Choice{0, t, 1, 4, nb});
            if (d.k > 32) out.push_back(Choice{8, t, 1, 4, nb});
          }
      }
  }
  return out;
}

}  // namespace

extern "C" {

int fgb_plan_create(fgb_ctx* ctx, const fgb_plan_desc* desc, int32_t tune_reps, fgb_plan** out) {
  if (!ctx || !desc || !out || !desc->A) return set_error(FGB_EINVAL, "fgb_plan_create: null argument");
  *out = nullptr;
  int rc = check_sparse(desc->A, "fgb_plan_create: A", true);
  if (rc) return rc;
  if (desc->op < FGB_PLAN_SPMV || desc->op > FGB_PLAN_SDDMM)
    return set_error(FGB_EINVAL, "fgb_plan_create: unknown op %d", desc->op);
  fgb_plan* p = new fgb_plan();
  p->ctx = ctx;
  p->d = *desc;
  p->A = *desc->A;
  p->d.A = &p->A;
  cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete p;
    return set_error(FGB_ECUDA, "fgb_plan_create: %s", cudaGetErrorString(e));
  }
  std::vector<Choice> cands = candidates(p);
  // scratch for the SpMM merge schedules: the largest any candidate needs
  if (p->d.op == FGB_PLAN_SPMM) {
    const size_t esz = p->d.dtype == FGB_F64 ? 8 : 4;
    for (const Choice& c : cands)
      if (c.path > 0 && c.variant < 2)  // the merge-path schedules
        p->scratch_bytes = std::max(p->scratch_bytes,
                                    spmm_merge_scratch_bytes(p->A.nrows, p->A.nnz, p->d.k, esz, c.path));
    if (p->scratch_bytes) {
      e = cudaMalloc(&p->scratch, p->scratch_bytes);
      if (e != cudaSuccess) {
        fgb_plan_destroy(p);
        return set_error(FGB_ENOMEM, "fgb_plan_create: scratch: %s", cudaGetErrorString(e));
      }
    }
  }
  const std::string key = tune_key(&p->d);
  Choice best = cands.front();
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_load_locked();
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      for (const Choice& c : cands)
        if (same_choice(c, it->second)) {
          best = c;
          cached = true;
        }
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_ms = -1.0, first_ms = -1.0;
  if (!cached && tune_reps > 0 && cands.size() > 1) {
    for (const Choice& c : cands) {
      rc = issue(p, c, p->stream, false);  // warm-up (and the item plan)
      if (rc) break;
      cudaEventRecord(e0, p->stream);
      for (int r = 0; r < tune_reps && rc == FGB_OK; ++r) rc = issue(p, c, p->stream, true);
      cudaEventRecord(e1, p->stream);
      if (rc) break;
      if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
        rc = set_error(FGB_ECUDA, "fgb_plan_create: timing: %s", cudaGetErrorString(e));
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= tune_reps;
      tune_log(key, c, ms);
      if (first_ms < 0) first_ms = ms;
      if (best_ms < 0 || ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (rc == FGB_OK) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      tune_cache_store_locked(key, best);
    }
  }
  if (rc == FGB_OK) {
    // matrix-only precomputation (merge-path items), then capture the rest
    rc = issue(p, best, p->stream, false);
    if (rc == FGB_OK && (e = cudaStreamSynchronize(p->stream)) != cudaSuccess)
      rc = set_error(FGB_ECUDA, "fgb_plan_create: %s", cudaGetErrorString(e));
  }
  if (rc == FGB_OK) {
    e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = issue(p, best, p->stream, true);
      cudaError_t e2 = cudaStreamEndCapture(p->stream, &p->graph);
      if (rc == FGB_OK && e2 != cudaSuccess)
        rc = set_error(FGB_ECUDA, "fgb_plan_create: capture: %s", cudaGetErrorString(e2));
      if (rc == FGB_OK && (e2 = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess)
        rc = set_error(FGB_ECUDA, "fgb_plan_create: instantiate: %s", cudaGetErrorString(e2));
    } else {
      rc = set_error(FGB_ECUDA, "fgb_plan_create: begin capture: %s", cudaGetErrorString(e));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    fgb_plan_destroy(p);
    return rc;
  }
  p->choice = best;
  for (auto it = p->vrows.begin(); it != p->vrows.end();) {  // and the chosen schedule
    const bool vrow_choice = p->d.op == FGB_PLAN_SPMM ? (best.variant == 2 || best.variant == 3)
                                                       : (best.variant == 3 || best.variant == 4);
    if (!vrow_choice || it->first != std::make_pair(best.path, best.bands)) {
      vrow_free(&it->second);
      it = p->vrows.erase(it);
    } else {
      ++it;
    }
  }
  for (auto it = p->panels.begin(); it != p->panels.end();) {  // keep only the chosen layout
    if (it->first != best.panels) {
      fgb_panels_destroy(it->second);
      it = p->panels.erase(it);
    } else {
      ++it;
    }
  }
  p->info.lanes = best.lanes;
  p->info.bands = best.bands;
  p->info.panels = best.panels;
  p->info.variant = best.variant;
  p->info.path = best.path;
  p->info.tuned_ms = best_ms;
  p->info.first_candidate_ms = first_ms;
  p->info.candidates = (int32_t)cands.size();
  p->info.from_cache = cached ? 1 : 0;
  p->info.launches = 0;  // kernel nodes of the captured graph: the launches of one execute
  size_t nn = 0;
  if (p->graph && cudaGraphGetNodes(p->graph, nullptr, &nn) == cudaSuccess && nn > 0) {
    std::vector<cudaGraphNode_t> nodes(nn);
    if (cudaGraphGetNodes(p->graph, nodes.data(), &nn) == cudaSuccess)
      for (size_t k = 0; k < nn; ++k) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++p->info.launches;
      }
  }
  *out = p;
  return FGB_OK;
}

int fgb_plan_execute(fgb_plan* p, void* stream) {
  if (!p || !p->exec) return set_error(FGB_EINVAL, "fgb_plan_execute: null plan");
  FGB_CUDA_TRY(cudaGraphLaunch(p->exec, pick_stream(p->ctx, stream)));
  return FGB_OK;
}

int fgb_plan_info_get(fgb_plan* p, fgb_plan_info* out) {
  if (!p || !out) return set_error(FGB_EINVAL, "fgb_plan_info_get: null argument");
  *out = p->info;
  return FGB_OK;
}

int fgb_plan_destroy(fgb_plan* p) {
  if (!p) return FGB_OK;
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->scratch) cudaFree(p->scratch);
  if (p->partial) cudaFree(p->partial);
  for (auto& kv : p->vrows) vrow_free(&kv.second);
  for (auto& kv : p->panels) fgb_panels_destroy(kv.second);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return FGB_OK;
}

}  // extern "C"
