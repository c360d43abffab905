// C ABI of the engine (include/fastpart.h): contexts, resident instances,
// validation of the hypergraph, uploads, kernel launches, read-backs.

#include "fp_internal.h"
#include "fp_device.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <chrono>
#include <new>
#include <vector>
#include <algorithm>
#include <memory>

namespace fp {
size_t refine_smem_bytes(int metric, int K);
cudaError_t launch_refine(const DevInstance& I, int passes, cudaStream_t st);
size_t metrics_scratch_bytes(int K);
cudaError_t launch_spec_ldg(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                            int* grid_out);
cudaError_t launch_spec_msg(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                            int* grid_out);
cudaError_t launch_spec_cn(const DevInstance& I, const SpecBuf& B, int passes, int num_sms, cudaStream_t st,
                           int* grid_out);
size_t spec_ldg_smem_bytes(int K);
size_t stream_smem_bytes(int K);
cudaError_t launch_stream_ldg(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, int num_sms,
                              cudaStream_t st);
size_t stream_msg_smem_bytes(int K);
cudaError_t launch_stream_msg(const DevInstance& I, const SpecBuf& B, const StreamArgs& S, int num_sms,
                              cudaStream_t st);
size_t spec_msg_smem_bytes(int K);
int create_inverse_device(int device, cudaStream_t st, int num_sms, int nov, int noe, long long pins,
                          const uint32_t* vptr_h, const uint32_t* vnets_h, uint32_t* nptr_h, uint32_t* npins_h);
int thin_nets_device(int device, cudaStream_t st, int num_sms, const fp_hypergraph* h, double size_lim,
                     int thin_min, HostGraph& out);
int bfs_order_device(int device, cudaStream_t st, int num_sms, const fp_hypergraph* h, int start, int* ordering,
                     int* far_out);
// The speculative grid-wide engine covers every metric as long as its shared
// memory fits a CTA (per-warp K-sized arrays) and the walked positions (vertices;
// nets for CN) stay below 2^28, the range of its cut words (position << 3 |
// reason); otherwise the single-CTA walk refines (same results).
constexpr int kMaxSpecPositions = 1 << 28;
static bool spec_supported(int metric, int K, int max_smem, int nov, int noe) {
  if (metric < FP_METRIC_CN || metric > FP_METRIC_MSRV) return false;
  if ((metric == FP_METRIC_CN ? noe : nov) >= kMaxSpecPositions) return false;
  const size_t static_smem = 8192;   // the kernels' static shared arrays, with room to spare
  if (metric == FP_METRIC_TM || metric == FP_METRIC_MSM)
    return spec_msg_smem_bytes(K) + static_smem <= (size_t)max_smem;
  if (metric == FP_METRIC_CN) return true;
  return spec_ldg_smem_bytes(K) + static_smem <= (size_t)max_smem;
}
// LDG metrics: vertex classes by work = sum over its nets of min(net size, K),
// the list slots an evaluation reads at most.  Light: one warp; medium: one CTA;
// above the super bound (or with 65536 nets or more, the limit of the candidate
// encoding): all warps of the grid, all inside the window.  Windows that end
// often (MSV moves nearly every vertex) favour a lower super bound, long ones
// (TV, MSM) a higher one; bounds from a sweep on the 4M-vertex Zipf workload.
// TM and MSM use the same classes in id order.
constexpr int kLightWork = 2048;
constexpr int kCnLightPins = 128;   // CN: nets with more pins are evaluated by one CTA,
constexpr int kCnGridPins = 1024;   //     with more than this by the whole grid
int default_super_work(int metric) {
  switch (metric) {
    case FP_METRIC_MSV: return 16384;
    case FP_METRIC_MSRV: return 32768;
    // measured on the 4M-vertex Zipf workload: passes 2-3 at 84 / 77 ms
    // against 94 / 90 with 32768 (pass 1 152 against 140)
    case FP_METRIC_TM: return 65536;
    default: return 262144;
  }
}
// Whole-grid vertices one window may hold.  Each one past the window's
// eventual cut (first mover for TM / MSM) is evaluated again in a later window,
// so metrics whose windows end early hold fewer.
int default_grid_verts(int metric) {
  switch (metric) {
    case FP_METRIC_TV:
    case FP_METRIC_CN:
    case FP_METRIC_MSM: return kMaxGridVerts;
    case FP_METRIC_TM:
    case FP_METRIC_MSRV: return 4;
    default: return 2;
  }
}
constexpr int kMaxSpecWarps = 16384;
cudaError_t launch_metrics(const DevInstance& I, void* scratch, long long* out, int num_sms, cudaStream_t st,
                           int* launches);
}  // namespace fp

using namespace fp;

struct fp_ctx {
  int device = 0;
  int num_sms = 0;    // SMs the engines size their grids for (fp_ctx_set_sm_limit)
  int dev_sms = 0;    // SMs of the device
  int max_smem = 0;   // opt-in shared memory per CTA
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  // fp_ctx_set_arena: one device allocation that instances of this context
  // take their buffers from, and pinned host words they share, so that
  // creating and releasing an instance calls neither cudaMalloc nor cudaFree
  // (which waits for the whole device, other contexts' work included)
  unsigned char* arena = nullptr;
  size_t arena_bytes = 0;
  size_t arena_used = 0;
  bool arena_busy = false;   // an instance holds the arena (one at a time)
  long long* h_moves = nullptr;     // pinned, with the arena
  int* h_status = nullptr;
  long long* h_metrics = nullptr;
};

struct fp_instance {
  fp_ctx* ctx = nullptr;
  HostGraph g;                 // host copy (validated)
  Problem pb;
  HostState st;
  bool has_state = false;
  DevInstance d{};
  std::vector<void*> allocs;
  long long dev_bytes = 0;        // bytes of the device allocations in `allocs`
  bool in_arena = false;          // buffers taken from ctx->arena (nothing in allocs)
  void* metric_scratch = nullptr;
  long long* metric_out = nullptr;
  long long* h_moves = nullptr;   // pinned
  int* h_status = nullptr;        // pinned
  long long* h_metrics = nullptr; // pinned
  int last_passes = 0;
  long long last_launches = 0;
  int engine = FP_ENGINE_AUTO;
  unsigned fault_leave_at = 0;    // fp_debug_barrier_fault: test hooks of the grid barrier
  unsigned fault_poll_limit = 0;
  int4* recs = nullptr;           // fp_set_decision_log: one record per vertex (net for CN)
  bool recs_valid = false;        // the last fp_refine wrote them
  SpecBuf sb{};
  int last_grid = 0;
  std::vector<int> heavy_pos;     // whole-grid-round vertices, by position in visiting order
  int* heavy_pos_d = nullptr;
  std::vector<int> mid_pos;       // CTA-evaluated vertices, by position
  int* mid_pos_d = nullptr;
  std::vector<int> porder;        // LDG engine positions (SpecBuf::porder)
  int* porder_d = nullptr;
  int* iso_list_d = nullptr;
  int* iso_before_d = nullptr;
  int* st_porder_d = nullptr;     // device stream positions, vertices without nets, their
  int* st_iso_d = nullptr;        //   counts before each position, whole-grid positions,
  int* st_before_d = nullptr;     //   last position that saw each part
  int* st_heavy_d = nullptr;
  int* st_mid_d = nullptr;
  unsigned char* st_class_d = nullptr;
  uint32_t* st_rec_d = nullptr;   // TM / MSM stream: (vertex, net) records
  uint32_t* st_prow_d = nullptr;  //   conn > 0 by row and by column
  uint32_t* st_pcol_d = nullptr;
  int* st_rowpos_d = nullptr;     //   first positions per row / column
  int* st_colpos_d = nullptr;
  int* st_saved_d = nullptr;      //   messages saved per part, per window offset
  uint32_t* st_actm_d = nullptr;  //   active / own-net part masks per window offset
  uint32_t* st_ownm_d = nullptr;
  int st_msg_wmax = 0;
  int* mark_pos_d = nullptr;
  StreamArgs sa{};                // device stream (TV / MSV / MSRV), csrc/fp_stream.cu
  bool stream_dev = false;        // the instance qualifies for the device stream
  int stream_mode = 0;            // fp_set_stream_mode: 0 auto, 1 host, 2 device where it qualifies
  bool last_stream_dev = false;   // the last fp_initial_partition ran on the device
  unsigned char* vclass_d = nullptr;
};

namespace {

const int kMaxPasses = 4096;
const int kSpecWindow = 16384;   // longest speculative window (vertices)
const int kMsgWindow = 65536;    // longest TM / MSM window
// Longest window of the TM / MSM device stream: its saved-message rows take K
// ints per window offset.
static int msg_stream_window(int nov) { return std::min(kSpecWindow, std::max(256, nov)); }

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return FP_OK;
  if (e == cudaErrorMemoryAllocation) return FP_ERR_NOMEM;
  return FP_ERR_CUDA;
}

// Arena allocations are 256-byte aligned, like cudaMalloc's.
constexpr size_t kArenaAlign = 256;

template <class T>
int dalloc(fp_instance* in, T** p, size_t n) {
  const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  if (in->in_arena) {
    fp_ctx* c = in->ctx;
    const size_t at = (c->arena_used + kArenaAlign - 1) & ~(kArenaAlign - 1);
    if (at + bytes > c->arena_bytes) return FP_ERR_NOMEM;
    c->arena_used = at + bytes;
    in->dev_bytes += (long long)bytes;
    *p = reinterpret_cast<T*>(c->arena + at);
    return FP_OK;
  }
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return cuda_status(e);
  in->allocs.push_back(q);
  in->dev_bytes += (long long)bytes;
  *p = static_cast<T*>(q);
  return FP_OK;
}

// Structural checks the kernels rely on: consistent CSRs (the net -> pins CSR is
// a permutation of the transpose of vertex -> nets), distinct pins per net,
// every net non-empty with its source among its pins, a permutation ordering.
int validate(const fp_hypergraph* h) {
  if (!h || h->nov <= 0 || h->noe < 0 || h->pins < 0 || h->pins >= (1ll << 31)) return FP_ERR_INVALID;
  if (!h->vptr || !h->nptr || !h->src || (h->pins > 0 && (!h->vnets || !h->npins))) return FP_ERR_INVALID;
  const int nov = h->nov, noe = h->noe;
  if (h->vptr[0] != 0 || h->nptr[0] != 0) return FP_ERR_INVALID;
  if ((long long)h->vptr[nov] != h->pins || (long long)h->nptr[noe] != h->pins) return FP_ERR_INVALID;
  for (int v = 0; v < nov; v++)
    if (h->vptr[v + 1] < h->vptr[v]) return FP_ERR_INVALID;
  for (int e = 0; e < noe; e++)
    if (h->nptr[e + 1] <= h->nptr[e]) return FP_ERR_INVALID;  // empty nets are rejected
  std::vector<uint32_t> cnt(noe, 0);
  for (long long k = 0; k < h->pins; k++) {
    if (h->vnets[k] >= (uint32_t)noe) return FP_ERR_INVALID;
    cnt[h->vnets[k]]++;
  }
  for (int e = 0; e < noe; e++)
    if (cnt[e] != h->nptr[e + 1] - h->nptr[e]) return FP_ERR_INVALID;
  // stamp[v] = e marks v as a pin of e according to vertex -> nets.
  std::vector<uint32_t> tptr(noe + 1, 0), tpins(h->pins);
  for (int e = 0; e < noe; e++) tptr[e + 1] = tptr[e] + cnt[e];
  std::vector<uint32_t> fill(tptr.begin(), tptr.end() - 1);
  for (int v = 0; v < nov; v++)
    for (uint32_t k = h->vptr[v]; k < h->vptr[v + 1]; k++) tpins[fill[h->vnets[k]]++] = (uint32_t)v;
  std::vector<int> stamp(nov, -1);
  for (int e = 0; e < noe; e++) {
    for (uint32_t k = tptr[e]; k < tptr[e + 1]; k++) {
      if (stamp[tpins[k]] == e) return FP_ERR_INVALID;  // vertex lists the net twice
      stamp[tpins[k]] = e;
    }
    bool src_ok = false;
    for (uint32_t k = h->nptr[e]; k < h->nptr[e + 1]; k++) {
      const uint32_t u = h->npins[k];
      if (u >= (uint32_t)nov || stamp[u] != e) return FP_ERR_INVALID;
      stamp[u] = -2 - e;
      if ((int)u == h->src[e]) src_ok = true;
    }
    if (!src_ok) return FP_ERR_INVALID;
  }
  if (h->weights) {
    long long W = 0;
    for (int v = 0; v < nov; v++) {
      if (h->weights[v] < 0) return FP_ERR_INVALID;
      W += h->weights[v];
    }
    if (W >= (1ll << 31)) return FP_ERR_INVALID;
  }
  if (h->ordering) {
    std::vector<char> seen(nov, 0);
    for (int z = 0; z < nov; z++) {
      const int v = h->ordering[z];
      if (v < 0 || v >= nov || seen[v]) return FP_ERR_INVALID;
      seen[v] = 1;
    }
  }
  return FP_OK;
}

int upload_state(fp_instance* in) {
  const HostState& st = in->st;
  cudaStream_t s = in->ctx->stream;
  const DevInstance& d = in->d;
  const int K = in->pb.K;
  cudaError_t e = cudaSuccess;
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  cp(d.part_vec, st.part_vec.data(), sizeof(int) * st.part_vec.size());
  cp(d.ep_len, st.ep_len.data(), sizeof(int) * st.ep_len.size());
  cp(d.ep_part, st.ep_part.data(), sizeof(int) * st.ep_part.size());
  cp(d.ep_cnt, st.ep_cnt.data(), sizeof(int) * st.ep_cnt.size());
  cp(d.part_sizes, st.part_sizes.data(), sizeof(int) * K);
  cp(d.marker, st.marker.data(), sizeof(int) * K);
  cp(d.send, st.send.data(), sizeof(int) * K);
  cp(d.recv, st.recv.data(), sizeof(int) * K);
  cp(d.msgs, st.msgs.data(), sizeof(int) * K);
  std::vector<uint32_t> zr, zc, c1r, c1c;
  if (in->pb.metric == FP_METRIC_TM || in->pb.metric == FP_METRIC_MSM) {
    const int words = (K + 31) / 32;
    zr.assign((size_t)K * words, 0);
    zc.assign((size_t)K * words, 0);
    c1r.assign((size_t)K * words, 0);
    c1c.assign((size_t)K * words, 0);
    for (int a = 0; a < K; a++)
      for (int b = 0; b < K; b++) {
        const int c = st.conn[(size_t)a * K + b];
        if (c == 0) {
          zr[(size_t)a * words + (b >> 5)] |= 1u << (b & 31);
          zc[(size_t)b * words + (a >> 5)] |= 1u << (a & 31);
        } else if (c == 1) {
          c1r[(size_t)a * words + (b >> 5)] |= 1u << (b & 31);
          c1c[(size_t)b * words + (a >> 5)] |= 1u << (a & 31);
        }
      }
    cp(d.conn, st.conn.data(), sizeof(int) * st.conn.size());
    cp(d.zrow, zr.data(), sizeof(uint32_t) * zr.size());
    cp(d.zcol, zc.data(), sizeof(uint32_t) * zc.size());
    cp(d.c1row, c1r.data(), sizeof(uint32_t) * c1r.size());
    cp(d.c1col, c1c.data(), sizeof(uint32_t) * c1c.size());
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // host vectors are pageable
  return cuda_status(e);
}

}  // namespace

extern "C" {

const char* fp_strerror(int status) {
  switch (status) {
    case FP_OK: return "ok";
    case FP_ERR_INVALID: return "invalid argument or malformed hypergraph";
    case FP_ERR_CUDA: return "CUDA runtime error";
    case FP_ERR_NOMEM: return "out of memory";
    case FP_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case FP_ERR_UNSUPPORTED: return "input on which the reference behaviour is undefined";
    case FP_ERR_STATE: return "call out of order";
    case FP_ERR_IO: return "file error";
    default: return "unknown status";
  }
}

int fp_validate(const fp_hypergraph* hg) {
  return fp::guarded([&]() -> int { return validate(hg); });
}

int fp_ctx_create(int32_t device, fp_ctx** out) {
  return fp::guarded([&]() -> int {
    if (!out) return FP_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return FP_ERR_CUDA;
    if (device < 0 || device >= n) return FP_ERR_INVALID;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_status(e);
    fp_ctx* c = new (std::nothrow) fp_ctx;
    if (!c) return FP_ERR_NOMEM;
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    c->dev_sms = c->num_sms;
    cudaDeviceGetAttribute(&c->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_status(e); }
    c->stream = c->own;
    *out = c;
    return FP_OK;
  });
}

static void arena_release(fp_ctx* c) {
  if (c->arena) cudaFree(c->arena);
  if (c->h_moves) cudaFreeHost(c->h_moves);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_metrics) cudaFreeHost(c->h_metrics);
  c->arena = nullptr;
  c->h_moves = nullptr;
  c->h_status = nullptr;
  c->h_metrics = nullptr;
  c->arena_bytes = c->arena_used = 0;
}

int fp_ctx_destroy(fp_ctx* ctx) {
  return fp::guarded([&]() -> int {
    if (!ctx) return FP_ERR_INVALID;
    cudaSetDevice(ctx->device);
    arena_release(ctx);
    if (ctx->own) cudaStreamDestroy(ctx->own);
    delete ctx;
    return FP_OK;
  });
}

int fp_ctx_set_arena(fp_ctx* ctx, int64_t bytes) {
  return fp::guarded([&]() -> int {
    if (!ctx || bytes < 0) return FP_ERR_INVALID;
    if (ctx->arena_busy) return FP_ERR_STATE;
    cudaSetDevice(ctx->device);
    arena_release(ctx);
    if (bytes == 0) return FP_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (size_t)bytes);
    if (e != cudaSuccess) return cuda_status(e);
    ctx->arena = static_cast<unsigned char*>(p);
    ctx->arena_bytes = (size_t)bytes;
    if (cudaMallocHost(&ctx->h_moves, sizeof(long long) * kMaxPasses) != cudaSuccess ||
        cudaMallocHost(&ctx->h_status, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_metrics, sizeof(long long) * 8) != cudaSuccess) {
      arena_release(ctx);
      return FP_ERR_NOMEM;
    }
    return FP_OK;
  });
}

int fp_ctx_set_sm_limit(fp_ctx* ctx, int32_t sms) {
  return fp::guarded([&]() -> int {
    if (!ctx || sms < 0) return FP_ERR_INVALID;
    ctx->num_sms = sms == 0 ? ctx->dev_sms : std::min(sms, ctx->dev_sms);
    return FP_OK;
  });
}

int fp_ctx_set_stream(fp_ctx* ctx, void* stream) {
  return fp::guarded([&]() -> int {
    if (!ctx) return FP_ERR_INVALID;
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own;
    return FP_OK;
  });
}

// Claims (no claim: a value above every position) and both parities of the
// whole-grid tallies start clear for every speculative launch: a launch leaves
// the tallies of its last window with whole-grid vertices, and an aborted
// launch its claims, behind.
static cudaError_t clear_spec_scratch(const SpecBuf& b, int noe, int K, cudaStream_t s) {
  const size_t ne = (size_t)std::max(noe, 1);
  cudaError_t e = cudaMemsetAsync(b.claim_m, 0x7f, sizeof(int) * ne, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.claim_c, 0x7f, sizeof(int) * ne, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.mask_c, 0, sizeof(uint32_t) * ne, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hcnt, 0, sizeof(int) * 2 * kMaxGridVerts * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hfirst, 0xff, sizeof(unsigned long long) * 2 * kMaxGridVerts * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hgain, 0, sizeof(int) * 2 * kMaxGridVerts * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hloss, 0, sizeof(int) * 2 * kMaxGridVerts * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hadelta, 0, sizeof(int) * 2 * kMaxGridVerts * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.hmisc, 0, sizeof(int) * 16 * kMaxGridVerts, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.mlast, 0, sizeof(unsigned long long) * K, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.mcnt, 0, sizeof(int) * 2, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b.ctab_over, 0, sizeof(int) * 2, s);
  if (e == cudaSuccess && b.ctab_mask) {
    const size_t n = (size_t)b.ctab_mask + 1;
    e = cudaMemsetAsync(b.ctab_key, 0xff, sizeof(unsigned long long) * n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.ctab_pos, 0x7f, sizeof(int) * n, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.ctab_cnt, 0, sizeof(int) * n, s);
  }
  return e;
}

// Positions of the device stream (TV, MSV, MSRV, CN; csrc/fp_stream.cu): the
// vertices with nets in visiting order, when every vertex without nets weighs
// 0 (those are placed from the sizes alone), and the positions whose vertex
// the whole grid places.  Sets stream_dev when the instance qualifies.
static int build_stream_positions(fp_instance* in) {
  const HostGraph& g = in->g;
  const Problem& pb = in->pb;
  std::vector<int> sp, siso, sbefore, heavy, mid;
  std::vector<unsigned char> pclass;
  // TM / MSM: one CTA places a vertex with many nets alone; the others: one
  // CTA evaluates a position with long lists, the grid places the longest
  const bool msgm = pb.metric == FP_METRIC_TM || pb.metric == FP_METRIC_MSM;
  bool w0 = true;
  for (int v = 0; v < g.nov; v++)
    if (g.vptr[v + 1] == g.vptr[v] && pb.w[v] != 0) w0 = false;
  for (int z = 0; z < g.nov; z++) {
    const int v = pb.order[z];
    if (g.vptr[v + 1] == g.vptr[v]) {
      siso.push_back(v);
      continue;
    }
    const uint32_t deg = g.vptr[v + 1] - g.vptr[v];
    if (msgm) {
      if (deg >= (uint32_t)kMsgStreamCta) heavy.push_back((int)sp.size());
    } else {
      // the list entries its evaluation reads at most: sum of min(|e|, K)
      long long work = 0;
      for (uint32_t i = g.vptr[v]; i < g.vptr[v + 1]; i++) {
        const int e = (int)g.vnets[i];
        work += std::min<long long>(g.nptr[e + 1] - g.nptr[e], pb.K);
      }
      unsigned char c = 0;
      if (deg >= (uint32_t)kStreamHeavy || work >= kStreamGridWork) {
        c = 2;
        heavy.push_back((int)sp.size());
      } else if (work >= kStreamCtaWork) {
        c = 1;
        mid.push_back((int)sp.size());
      }
      pclass.push_back(c);
    }
    sp.push_back(v);
    sbefore.push_back((int)siso.size());
  }
  sbefore.push_back((int)siso.size());
  in->stream_dev = w0 && !sp.empty() && pb.K <= kStreamMaxK &&
                   (msgm ? stream_msg_smem_bytes(pb.K) : stream_smem_bytes(pb.K)) + 4096 <= (size_t)in->ctx->max_smem;
  in->sa.porder = in->st_porder_d;
  in->sa.npos = (int)sp.size();
  in->sa.iso_list = in->st_iso_d;
  in->sa.iso_before = in->st_before_d;
  in->sa.niso = (int)siso.size();
  in->sa.heavy_pos = in->st_heavy_d;
  in->sa.nheavy = (int)heavy.size();
  in->sa.mid_pos = in->st_mid_d;
  in->sa.nmid = (int)mid.size();
  in->sa.pclass = in->st_class_d;
  in->sa.mark_pos = in->mark_pos_d;
  // the slot records: CN's refinement scratch of (pin, offset) pairs is free
  // before the first refinement
  in->sa.rec = pb.metric == FP_METRIC_CN ? reinterpret_cast<uint32_t*>(in->sb.cn_moved)
               : msgm                       ? in->st_rec_d
                                            : in->sb.rec;
  in->sa.prow = in->st_prow_d;
  in->sa.pcol = in->st_pcol_d;
  in->sa.rowpos = in->st_rowpos_d;
  in->sa.colpos = in->st_colpos_d;
  in->sa.saved = in->st_saved_d;
  in->sa.actm = in->st_actm_d;
  in->sa.ownm = in->st_ownm_d;
  in->sa.msg_wmax = msg_stream_window(g.nov);
  // Walking the changed decisions of a window on one warp (instead of ending
  // the window at the first) pays where most windows end at a change: CN
  // 8.9 -> 3.3 s on the 4M-vertex Zipf workload; the LDG streams, whose
  // windows end at conflicts as often, went 1.05 -> 1.33 s, so they cut.
  in->sa.walk = pb.metric == FP_METRIC_CN ? 1 : 0;
  cudaStream_t s0 = in->ctx->stream;
  cudaError_t e0 = cudaSuccess;
  if (in->stream_dev) {
    e0 = cudaMemcpyAsync(in->st_porder_d, sp.data(), sizeof(int) * sp.size(), cudaMemcpyHostToDevice, s0);
    if (e0 == cudaSuccess && !siso.empty())
      e0 = cudaMemcpyAsync(in->st_iso_d, siso.data(), sizeof(int) * siso.size(), cudaMemcpyHostToDevice, s0);
    if (e0 == cudaSuccess)
      e0 = cudaMemcpyAsync(in->st_before_d, sbefore.data(), sizeof(int) * sbefore.size(), cudaMemcpyHostToDevice,
                           s0);
    if (e0 == cudaSuccess && !heavy.empty())
      e0 = cudaMemcpyAsync(in->st_heavy_d, heavy.data(), sizeof(int) * heavy.size(), cudaMemcpyHostToDevice, s0);
    if (e0 == cudaSuccess && !mid.empty())
      e0 = cudaMemcpyAsync(in->st_mid_d, mid.data(), sizeof(int) * mid.size(), cudaMemcpyHostToDevice, s0);
    if (e0 == cudaSuccess && !pclass.empty())
      e0 = cudaMemcpyAsync(in->st_class_d, pclass.data(), pclass.size(), cudaMemcpyHostToDevice, s0);
    if (e0 == cudaSuccess) e0 = cudaStreamSynchronize(s0);
  }
  return cuda_status(e0);
}

// Positions of the LDG engine (TV / MSV / MSRV).  A vertex without nets and
// with weight 0 reads only the part sizes and changes nothing that a later
// decision reads; for TV, when every vertex without nets weighs 0 (vertex
// weight = degree), they are left out of the walked positions and decided
// after each window from the exact sizes at their place.  Uploads porder, iso_list and
// iso_before and fills the SpecBuf fields.
static int build_positions(fp_instance* in) {
  const HostGraph& g = in->g;
  const Problem& pb = in->pb;
  in->porder.clear();
  std::vector<int> iso, before;
  bool compact = true, any_iso = false;
  for (int v = 0; v < g.nov; v++)
    if (g.vptr[v + 1] == g.vptr[v]) {
      any_iso = true;
      if (pb.w[v] != 0) compact = false;
    }
  // Measured on the 4M-vertex Zipf workload (degree weights): TV 75 -> 48 ms
  // per pass; MSV unchanged and MSRV slower (430 vs 318 ms), because their
  // windows end every few dozen positions (max-volume changes, in-window
  // fixes) and a window of compacted positions wastes more evaluations past
  // its cut -- so only TV walks compacted positions.
  compact = compact && any_iso && pb.metric == FP_METRIC_TV;
  for (int z = 0; z < g.nov; z++) {
    const int v = pb.order[z];
    if (compact && g.vptr[v + 1] == g.vptr[v]) {
      iso.push_back(v);
    } else {
      in->porder.push_back(v);
      before.push_back((int)iso.size());
    }
  }
  if (compact && in->porder.empty()) {   // nothing but vertices without nets: walk them all
    in->porder.assign(pb.order.begin(), pb.order.end());
    iso.clear();
    before.clear();
    compact = false;
  }
  before.push_back((int)iso.size());
  in->sb.porder = in->porder_d;
  in->sb.npos = (int)in->porder.size();
  in->sb.iso_list = in->iso_list_d;
  in->sb.iso_before = in->iso_before_d;
  in->sb.niso = compact ? (int)iso.size() : 0;
  cudaStream_t s = in->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(in->porder_d, in->porder.data(), sizeof(int) * in->porder.size(),
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !iso.empty())
    e = cudaMemcpyAsync(in->iso_list_d, iso.data(), sizeof(int) * iso.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && compact)
    e = cudaMemcpyAsync(in->iso_before_d, before.data(), sizeof(int) * before.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // host vectors are local
  return cuda_status(e);
}

// Vertex classes of the LDG engine (see kLightWork) and the position lists of
// the medium and whole-grid vertices, uploaded to the device.
static int classify(fp_instance* in, long long light_work, long long super_work) {
  const HostGraph& g = in->g;
  const Problem& pb = in->pb;
  std::vector<unsigned char> cls(g.nov, 0);
  in->heavy_pos.clear();
  in->mid_pos.clear();
  if (pb.metric == FP_METRIC_CN) {
    // CN walks the nets in id order (CN/partition.cpp:245); a net with more
    // than light_work pins is evaluated by a whole CTA, with more than
    // super_work by the whole grid
    const long long grid_pins = std::max(light_work, super_work);
    for (int e = 0; e < g.noe; e++) {
      const long long n = g.nptr[e + 1] - g.nptr[e];
      if (n > grid_pins) in->heavy_pos.push_back(e);
      else if (n > light_work) in->mid_pos.push_back(e);
    }
    in->sb.cn_big = (int)std::min<long long>(light_work, 0x7fffffff);
    in->sb.cn_grid = (int)std::min<long long>(grid_pins, 0x7fffffff);
    in->sb.nheavy = (int)in->heavy_pos.size();
    in->sb.nmid = (int)in->mid_pos.size();
    cudaError_t e = cudaSuccess;
    if (in->sb.nmid)
      e = cudaMemcpyAsync(in->mid_pos_d, in->mid_pos.data(), sizeof(int) * in->sb.nmid, cudaMemcpyHostToDevice,
                          in->ctx->stream);
    if (e == cudaSuccess && in->sb.nheavy)
      e = cudaMemcpyAsync(in->heavy_pos_d, in->heavy_pos.data(), sizeof(int) * in->sb.nheavy,
                          cudaMemcpyHostToDevice, in->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(in->ctx->stream);
    return cuda_status(e);
  }
  // TM and MSM walk the vertices in id order (TM/partition.cpp:300), the others
  // in the visiting order.
  const bool by_id = pb.metric == FP_METRIC_TM || pb.metric == FP_METRIC_MSM;
  const int npos = by_id ? g.nov : (int)in->porder.size();
  for (int z = 0; z < npos; z++) {
    const int v = by_id ? z : in->porder[z];
    long long work = 0;
    for (uint32_t k = g.vptr[v]; k < g.vptr[v + 1]; k++) {
      const uint32_t e = g.vnets[k];
      work += std::min<long long>(g.nptr[e + 1] - g.nptr[e], pb.K);
    }
    const long long deg = g.vptr[v + 1] - g.vptr[v];
    if (work > super_work || deg >= 65536) {
      cls[v] = 2;
      in->heavy_pos.push_back(z);
    } else if (work > light_work) {
      cls[v] = 1;
      in->mid_pos.push_back(z);
    }
  }
  in->sb.nheavy = (int)in->heavy_pos.size();
  in->sb.nmid = (int)in->mid_pos.size();
  cudaStream_t s = in->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(in->vclass_d, cls.data(), g.nov, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && in->sb.nheavy)
    e = cudaMemcpyAsync(in->heavy_pos_d, in->heavy_pos.data(), sizeof(int) * in->sb.nheavy, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && in->sb.nmid)
    e = cudaMemcpyAsync(in->mid_pos_d, in->mid_pos.data(), sizeof(int) * in->sb.nmid, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // host vectors are pageable and local
  return cuda_status(e);
}

int fp_instance_create(fp_ctx* ctx, const fp_hypergraph* h, int32_t K, int32_t metric, double eps_factor,
                       fp_instance** out) {
  // an exception releases the half-built instance (its device buffers included)
  fp_instance* made = nullptr;
  return fp::guarded([&]() -> int {
    if (!ctx || !out || metric < 0 || metric > 5 || K < 2 || K > kMaxK || !(eps_factor > 0)) return FP_ERR_INVALID;
    *out = nullptr;
    fp_instance* in = new (std::nothrow) fp_instance;
    if (!in) return FP_ERR_NOMEM;
    made = in;
    in->ctx = ctx;
    if (ctx->arena) {
      // the context's arena serves one instance at a time
      if (ctx->arena_busy) { delete in; made = nullptr; return FP_ERR_STATE; }
      in->in_arena = true;
      ctx->arena_busy = true;
      ctx->arena_used = 0;
    }
    int rc = make_problem(h, K, metric, eps_factor, in->g, in->pb);   // validates h
    if (rc) { fp_instance_destroy(in); made = nullptr; return rc; }
    const HostGraph& g = in->g;
    const Problem& pb = in->pb;

    cudaSetDevice(ctx->device);
    DevInstance& d = in->d;
    d.nov = g.nov;
    d.noe = g.noe;
    d.pins = g.pins;
    d.K = K;
    d.metric = metric;
    d.C = pb.C;
    d.max_pw = (int)(pb.xw + (pb.xw * 0.1));
    d.min_pw = (int)(pb.xw - (pb.xw * 0.1));
    const size_t KK = (size_t)K * K, words = (size_t)(K + 31) / 32;
    const bool msg = metric == FP_METRIC_TM || metric == FP_METRIC_MSM;
    const bool cn = metric == FP_METRIC_CN;
    const bool ldg = !msg && !cn;
    const bool vfix = metric == FP_METRIC_MSV || metric == FP_METRIC_MSRV;   // in-window decision fixes
    // exact count claims of the LDG engine: a table well above the entries of a
    // round (two per count-only net of a window's movers)
    size_t ctab = 4096;
    while (ctab < (size_t)2 * g.noe && ctab < ((size_t)1 << 21)) ctab <<= 1;
    uint32_t *vptr, *vnets, *nptr, *npins;
    int *src, *w, *order;
    if ((rc = dalloc(in, &vptr, g.nov + 1)) || (rc = dalloc(in, &vnets, g.pins)) || (rc = dalloc(in, &nptr, g.noe + 1)) ||
        (rc = dalloc(in, &npins, g.pins)) || (rc = dalloc(in, &src, g.noe)) || (rc = dalloc(in, &w, g.nov)) ||
        (rc = dalloc(in, &order, g.nov)) || (rc = dalloc(in, &d.part_vec, g.nov)) || (rc = dalloc(in, &d.ep_len, g.noe)) ||
        (rc = dalloc(in, &d.ep_part, g.pins)) || (rc = dalloc(in, &d.ep_cnt, g.pins)) ||
        (rc = dalloc(in, &d.part_sizes, K)) || (rc = dalloc(in, &d.marker, K)) || (rc = dalloc(in, &d.send, K)) ||
        (rc = dalloc(in, &d.recv, K)) || (rc = dalloc(in, &d.msgs, K)) || (rc = dalloc(in, &d.conn, msg ? KK : 1)) ||
        (rc = dalloc(in, &d.zrow, msg ? K * words : 1)) || (rc = dalloc(in, &d.zcol, msg ? K * words : 1)) ||
        (rc = dalloc(in, &d.c1row, msg ? K * words : 1)) || (rc = dalloc(in, &d.c1col, msg ? K * words : 1)) ||
        (rc = dalloc(in, &d.moves, kMaxPasses)) || (rc = dalloc(in, &d.status, 1)) ||
        (rc = dalloc(in, &in->sb.ctl, 8)) || (rc = dalloc(in, &in->sb.bar, 4)) || (rc = dalloc(in, &in->sb.stats, kNumStats)) || (rc = dalloc(in, &in->sb.dec, std::max(kSpecWindow, kMsgWindow))) ||
        (rc = dalloc(in, &in->sb.flag, kSpecWindow)) || (rc = dalloc(in, &in->sb.slack, kSpecWindow)) ||
        (rc = dalloc(in, &in->sb.vslack, kSpecWindow)) || (rc = dalloc(in, &in->sb.wt, kSpecWindow)) ||
        (rc = dalloc(in, &in->sb.vd, kSpecWindow)) || (rc = dalloc(in, &in->sb.scan, (size_t)kSpecWindow * words)) ||
        (rc = dalloc(in, &in->sb.rgain, std::max(kSpecWindow, kMsgWindow))) ||
        (rc = dalloc(in, &in->sb.rloss, std::max(kSpecWindow, kMsgWindow))) ||
        (rc = dalloc(in, &in->sb.rec, ldg ? g.pins : 1)) || (rc = dalloc(in, &in->sb.rec_slot, ldg ? g.pins : 1)) ||
        (rc = dalloc(in, &in->sb.ctab_key, ldg ? ctab : 1)) || (rc = dalloc(in, &in->sb.ctab_pos, ldg ? ctab : 1)) ||
        (rc = dalloc(in, &in->sb.ctab_cnt, ldg ? ctab : 1)) ||
        (rc = dalloc(in, &in->sb.ctab_over, 2)) || (rc = dalloc(in, &in->sb.dfix, kSpecWindow)) ||
        (rc = dalloc(in, &in->sb.rec_slot2, vfix ? g.pins : 1)) ||
        (rc = dalloc(in, &in->sb.cn_moved, cn ? g.pins : 1)) || (rc = dalloc(in, &in->sb.cn_kcnt, cn ? g.noe : 1)) ||
        (rc = dalloc(in, &in->sb.cn_nets, cn ? g.noe : 1)) || (rc = dalloc(in, &in->sb.cn_cnt, 4)) ||
        (rc = dalloc(in, &in->sb.cn_wit, cn ? g.nov : 1)) || (rc = dalloc(in, &in->vclass_d, g.nov)) ||
        (rc = dalloc(in, &in->sb.cand, (size_t)kSpecWindow * K)) || (rc = dalloc(in, &in->sb.ncand, kSpecWindow)) ||
        (rc = dalloc(in, &in->sb.mlist, kSpecWindow)) || (rc = dalloc(in, &in->sb.midx, kSpecWindow)) ||
        (rc = dalloc(in, &in->sb.mcnt, 2)) ||
        (rc = dalloc(in, &in->sb.wsum, kMaxSpecWarps)) || (rc = dalloc(in, &in->sb.vsum, kMaxSpecWarps)) ||
        (rc = dalloc(in, &in->sb.claim_m, g.noe)) || (rc = dalloc(in, &in->sb.claim64, g.noe)) || (rc = dalloc(in, &in->sb.claim_c, g.noe)) ||
        (rc = dalloc(in, &in->sb.mask_c, g.noe)) || (rc = dalloc(in, &in->sb.hcnt, 2 * kMaxGridVerts * K)) ||
        (rc = dalloc(in, &in->sb.hfirst, 2 * kMaxGridVerts * K)) ||
        (rc = dalloc(in, &in->sb.hgain, 2 * kMaxGridVerts * K)) ||
        (rc = dalloc(in, &in->sb.hloss, 2 * kMaxGridVerts * K)) ||
        (rc = dalloc(in, &in->sb.hadelta, 2 * kMaxGridVerts * K)) ||
        (rc = dalloc(in, &in->sb.hmisc, 16 * kMaxGridVerts)) || (rc = dalloc(in, &in->sb.mlast, K)) || (rc = dalloc(in, &in->heavy_pos_d, std::max(g.nov, g.noe))) ||
        (rc = dalloc(in, &in->mid_pos_d, std::max(g.nov, g.noe))) ||
        (rc = dalloc(in, &in->porder_d, ldg ? g.nov : 1)) || (rc = dalloc(in, &in->iso_list_d, ldg ? g.nov : 1)) ||
        (rc = dalloc(in, &in->iso_before_d, ldg ? g.nov + 1 : 1)) ||
        (rc = dalloc(in, &in->st_porder_d, g.nov)) || (rc = dalloc(in, &in->st_iso_d, g.nov)) ||
        (rc = dalloc(in, &in->st_before_d, g.nov + 1)) || (rc = dalloc(in, &in->st_heavy_d, g.nov)) ||
        (rc = dalloc(in, &in->st_mid_d, ldg || cn ? g.nov : 1)) ||
        (rc = dalloc(in, &in->st_class_d, ldg || cn ? g.nov : 1)) ||
        (rc = dalloc(in, &in->mark_pos_d, K)) ||
        (rc = dalloc(in, &in->st_rec_d, msg ? g.pins : 1)) || (rc = dalloc(in, &in->st_prow_d, msg ? K * words : 1)) ||
        (rc = dalloc(in, &in->st_pcol_d, msg ? K * words : 1)) ||
        (rc = dalloc(in, &in->st_rowpos_d, msg ? 2 * K : 1)) || (rc = dalloc(in, &in->st_colpos_d, msg ? 2 * K : 1)) ||
        (rc = dalloc(in, &in->st_saved_d, msg ? (size_t)msg_stream_window(g.nov) * K : 1)) ||
        (rc = dalloc(in, &in->st_actm_d, msg ? (size_t)msg_stream_window(g.nov) * words : 1)) ||
        (rc = dalloc(in, &in->st_ownm_d, msg ? (size_t)msg_stream_window(g.nov) * words : 1)) ||
        (rc = dalloc(in, &in->metric_out, 8))) {
      fp_instance_destroy(in);
      return rc;
    }
    void* ms = nullptr;
    cudaError_t e = cudaSuccess;
    if (in->in_arena) {
      unsigned char* q = nullptr;
      if ((rc = dalloc(in, &q, metrics_scratch_bytes(K)))) { fp_instance_destroy(in); return rc; }
      ms = q;
    } else {
      e = cudaMalloc(&ms, metrics_scratch_bytes(K));
      if (e != cudaSuccess) { fp_instance_destroy(in); return cuda_status(e); }
      in->allocs.push_back(ms);
      in->dev_bytes += (long long)metrics_scratch_bytes(K);
    }
    in->metric_scratch = ms;
    in->sb.wmax = kSpecWindow;
    in->sb.ctab_mask = ldg ? (unsigned)(ctab - 1) : 0u;
    in->sb.wmax_msg = kMsgWindow;
    in->sb.gmax = default_grid_verts(metric);
    // window regrowth after a cut: twice the last valid length for MSV (cuts
    // every few hundred positions), four times for the metrics with rarer cuts
    in->sb.wgrow = metric == FP_METRIC_MSV ? 2 : 4;
    // at least one position per warp of the grid after a cut: measured on the
    // 4M-vertex Zipf workload, MSRV 410 -> 355 ms per pass, MSV 912 -> 906,
    // TV unchanged (against 256)
    in->sb.wmin = 0;
    in->sb.maxfix = 32;
    in->sb.max_warps = kMaxSpecWarps;
    in->sb.heavy_pos = in->heavy_pos_d;
    in->sb.mid_pos = in->mid_pos_d;
    in->sb.vclass = in->vclass_d;
    {
      cudaStream_t s0 = ctx->stream;
      e = clear_spec_scratch(in->sb, g.noe, K, s0);
      if (e == cudaSuccess && cn) e = cudaMemsetAsync(in->sb.cn_wit, 0xff, sizeof(int) * g.nov, s0);   // no witnesses
      if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
      if (e != cudaSuccess) { fp_instance_destroy(in); return cuda_status(e); }
      if (ldg && (rc = build_positions(in))) { fp_instance_destroy(in); return rc; }
      if ((rc = build_stream_positions(in))) { fp_instance_destroy(in); return rc; }
      rc = classify(in, metric == FP_METRIC_CN ? kCnLightPins : kLightWork,
                    metric == FP_METRIC_CN ? kCnGridPins : default_super_work(metric));
      if (rc) { fp_instance_destroy(in); return rc; }
    }
    if (in->in_arena) {   // the context's pinned words
      in->h_moves = ctx->h_moves;
      in->h_status = ctx->h_status;
      in->h_metrics = ctx->h_metrics;
    } else if (cudaMallocHost(&in->h_moves, sizeof(long long) * kMaxPasses) != cudaSuccess ||
               cudaMallocHost(&in->h_status, sizeof(int)) != cudaSuccess ||
               cudaMallocHost(&in->h_metrics, sizeof(long long) * 8) != cudaSuccess) {
      fp_instance_destroy(in);
      return FP_ERR_NOMEM;
    }
    d.vptr = vptr; d.vnets = vnets; d.nptr = nptr; d.npins = npins; d.src = src; d.w = w; d.order = order;
    cudaStream_t s = ctx->stream;
    e = cudaMemcpyAsync(vptr, g.vptr.data(), sizeof(uint32_t) * (g.nov + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && g.pins) e = cudaMemcpyAsync(vnets, g.vnets.data(), sizeof(uint32_t) * g.pins, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(nptr, g.nptr.data(), sizeof(uint32_t) * (g.noe + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && g.pins) e = cudaMemcpyAsync(npins, g.npins.data(), sizeof(uint32_t) * g.pins, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && g.noe) e = cudaMemcpyAsync(src, g.src.data(), sizeof(int) * g.noe, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w, pb.w.data(), sizeof(int) * g.nov, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(order, pb.order.data(), sizeof(int) * g.nov, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.status, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { fp_instance_destroy(in); return cuda_status(e); }
    *out = in;
    return FP_OK;
  }, [&] {
    if (made) fp_instance_destroy(made);
    if (out) *out = nullptr;
  });
}

int fp_instance_device_bytes(fp_instance* in, int64_t* bytes) {
  return fp::guarded([&]() -> int {
    if (!in || !bytes) return FP_ERR_INVALID;
    *bytes = in->dev_bytes;
    return FP_OK;
  });
}

// The bytes fp_instance_create allocates on the device, from the sizes alone:
// the same buffers, element types and counts, in the same order.
int fp_instance_footprint(int32_t nov, int32_t noe, int64_t pins, int32_t K, int32_t metric, int64_t* bytes) {
  return fp::guarded([&]() -> int {
    if (!bytes || nov <= 0 || noe < 0 || pins < 0 || pins >= (1ll << 31) || metric < 0 || metric > 5 || K < 2 ||
        K > kMaxK)
      return FP_ERR_INVALID;
    const size_t KK = (size_t)K * K, words = (size_t)(K + 31) / 32;
    const bool msg = metric == FP_METRIC_TM || metric == FP_METRIC_MSM;
    const bool cn = metric == FP_METRIC_CN;
    const bool ldg = !msg && !cn;
    const bool vfix = metric == FP_METRIC_MSV || metric == FP_METRIC_MSRV;
    size_t ctab = 4096;
    while (ctab < (size_t)2 * noe && ctab < ((size_t)1 << 21)) ctab <<= 1;
    const size_t P = (size_t)pins, V = (size_t)nov, E = (size_t)noe, G2K = 2 * (size_t)kMaxGridVerts * K;
    const size_t W = kSpecWindow, VE = std::max(V, E);
    long long b = 0;
    auto add = [&b](size_t n, size_t elem) { b += (long long)(std::max<size_t>(n, 1) * elem); };
    // hypergraph, state
    add(V + 1, 4); add(P, 4); add(E + 1, 4); add(P, 4); add(E, 4); add(V, 4); add(V, 4);
    add(V, 4); add(E, 4); add(P, 4); add(P, 4);
    for (int k = 0; k < 5; k++) add(K, 4);                   // part_sizes, marker, send, recv, msgs
    add(msg ? KK : 1, 4);                                    // conn
    for (int k = 0; k < 4; k++) add(msg ? K * words : 1, 4);  // zero and conn == 1 masks
    add(kMaxPasses, 8); add(1, 4);                           // moves, status
    // speculation scratch
    add(8, 4); add(4, 4); add(kNumStats, 8); add(std::max(kSpecWindow, kMsgWindow), 4);
    add(W, 1); add(W, 4); add(W, 4); add(W, 4); add(W, 4);   // flag, slack, vslack, wt, vd
    add(W * words, 4);                                       // scan
    add(std::max(kSpecWindow, kMsgWindow), 4); add(std::max(kSpecWindow, kMsgWindow), 4);   // rgain, rloss
    add(ldg ? P : 1, 4); add(ldg ? P : 1, 8);                // rec, rec_slot
    add(ldg ? ctab : 1, 8); add(ldg ? ctab : 1, 4); add(ldg ? ctab : 1, 4);
    add(2, 4); add(W, 4);                                    // ctab_over, dfix
    add(vfix ? P : 1, 8);                                    // rec_slot2
    add(cn ? P : 1, 8); add(cn ? E : 1, 4); add(cn ? E : 1, 8); add(4, 4); add(cn ? V : 1, 4);
    add(V, 1);                                               // vertex classes
    add(W * K, 8); add(W, 4); add(W, 16); add(W, 4); add(2, 4);   // cand, ncand, mlist, midx, mcnt
    add(kMaxSpecWarps, 4); add(kMaxSpecWarps, 4);            // wsum, vsum
    add(E, 4); add(E, 8); add(E, 4); add(E, 4);              // claim_m, claim64, claim_c, mask_c
    add(G2K, 4); add(G2K, 8); add(G2K, 4); add(G2K, 4); add(G2K, 4);
    add(16 * (size_t)kMaxGridVerts, 4); add(K, 8);           // hmisc, mlast
    add(VE, 4); add(VE, 4);                                  // heavy / medium positions
    add(ldg ? V : 1, 4); add(ldg ? V : 1, 4); add(ldg ? V + 1 : 1, 4);   // porder, iso_list, iso_before
    add(V, 4); add(V, 4); add(V + 1, 4); add(V, 4);          // device stream: positions, iso, before,
                                                             //   whole-grid positions,
    add(ldg || cn ? V : 1, 4); add(ldg || cn ? V : 1, 1);   //   CTA positions, classes,
    add(K, 4);                                              //   mark_pos
    {
      const size_t mw = (size_t)msg_stream_window(nov);      //   TM / MSM: records, masks, first
      add(msg ? P : 1, 4); add(msg ? K * words : 1, 4); add(msg ? K * words : 1, 4);   //   positions,
      add(msg ? 2 * (size_t)K : 1, 4); add(msg ? 2 * (size_t)K : 1, 4);               //   saved messages,
      add(msg ? mw * K : 1, 4); add(msg ? mw * words : 1, 4); add(msg ? mw * words : 1, 4);   // part masks
    }
    add(8, 8);                                               // metric_out
    b += (long long)metrics_scratch_bytes(K);
    *bytes = b;
    return FP_OK;
  });
}

int fp_instance_destroy(fp_instance* in) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    cudaSetDevice(in->ctx->device);
    for (void* p : in->allocs) cudaFree(p);
    if (in->recs) cudaFree(in->recs);
    if (in->in_arena) {
      // the buffers stay in the context's arena for the next instance; its
      // work on the context's stream is ordered after this one's
      in->ctx->arena_busy = false;
      in->ctx->arena_used = 0;
    } else {
      if (in->h_moves) cudaFreeHost(in->h_moves);
      if (in->h_status) cudaFreeHost(in->h_status);
      if (in->h_metrics) cudaFreeHost(in->h_metrics);
    }
    delete in;
    return FP_OK;
  });
}

// The LDG metrics' stream on the device (csrc/fp_stream.cu); the result is
// copied back into the host state, which fp_reset_state uploads again.
static int device_stream(fp_instance* in) {
  cudaSetDevice(in->ctx->device);
  cudaStream_t s = in->ctx->stream;
  const HostGraph& g = in->g;
  const int K = in->pb.K;
  DevInstance& d = in->d;
  static const int none[8] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff,
                              0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
  cudaError_t e = cudaMemsetAsync(d.part_vec, 0xff, sizeof(int) * g.nov, s);
  auto zero = [&](void* p, size_t bytes, int val) {
    if (e == cudaSuccess && bytes) e = cudaMemsetAsync(p, val, bytes, s);
  };
  zero(d.ep_len, sizeof(int) * g.noe, 0);
  zero(d.ep_part, sizeof(int) * g.pins, 0xff);
  zero(d.ep_cnt, sizeof(int) * g.pins, 0);
  zero(d.part_sizes, sizeof(int) * K, 0);
  zero(d.marker, sizeof(int) * K, 0xff);
  zero(d.send, sizeof(int) * K, 0);
  zero(d.recv, sizeof(int) * K, 0);
  zero(d.msgs, sizeof(int) * K, 0);
  zero(d.status, sizeof(int), 0);
  zero(in->mark_pos_d, sizeof(int) * K, 0xff);
  zero(in->sb.claim64, sizeof(unsigned long long) * std::max(g.noe, 1), 0);
  zero(in->sb.bar, sizeof(unsigned) * 4, 0);
  zero(in->sb.stats, sizeof(unsigned long long) * kNumStats, 0);
  if (e == cudaSuccess) e = cudaMemcpyAsync(in->sb.ctl, none, sizeof(none), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = clear_spec_scratch(in->sb, g.noe, K, s);
  const bool msg = in->pb.metric == FP_METRIC_TM || in->pb.metric == FP_METRIC_MSM;
  std::vector<int> conn0;
  if (msg) {
    // connection counts start at 0 (MSM: -1 on the diagonal, MSM/partition.cpp:
    // 150-156); no entry is positive; no first positions
    const size_t words = (size_t)(K + 31) / 32;
    conn0.assign((size_t)K * K, 0);
    if (in->pb.metric == FP_METRIC_MSM)
      for (int i = 0; i < K; i++) conn0[(size_t)i * K + i] = -1;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d.conn, conn0.data(), sizeof(int) * conn0.size(), cudaMemcpyHostToDevice, s);
    zero(in->st_prow_d, sizeof(uint32_t) * K * words, 0);
    zero(in->st_pcol_d, sizeof(uint32_t) * K * words, 0);
    zero(in->st_rowpos_d, sizeof(int) * 2 * K, 0x7f);
    zero(in->st_colpos_d, sizeof(int) * 2 * K, 0x7f);
  }
  if (e == cudaSuccess)
    e = msg ? launch_stream_msg(d, in->sb, in->sa, in->ctx->num_sms, s)
            : launch_stream_ldg(d, in->sb, in->sa, in->ctx->num_sms, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(in->h_status, d.status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e);
  if (*in->h_status) return *in->h_status;
  HostState& st = in->st;
  st.part_vec.resize(g.nov);
  st.part_sizes.resize(K);
  st.ep_start.assign(g.nptr.begin(), g.nptr.end());
  st.ep_len.resize(g.noe);
  st.ep_part.resize(g.pins);
  st.ep_cnt.resize(g.pins);
  st.marker.resize(K);
  st.send.resize(K);
  st.recv.resize(K);
  st.msgs.assign(K, 0);
  st.conn.clear();
  if (msg) st.conn.resize((size_t)K * K);
  auto back = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  };
  if (msg) {
    back(st.conn.data(), d.conn, sizeof(int) * st.conn.size());
    back(st.msgs.data(), d.msgs, sizeof(int) * K);
  }
  back(st.part_vec.data(), d.part_vec, sizeof(int) * g.nov);
  back(st.part_sizes.data(), d.part_sizes, sizeof(int) * K);
  back(st.ep_len.data(), d.ep_len, sizeof(int) * g.noe);
  back(st.ep_part.data(), d.ep_part, sizeof(int) * g.pins);
  back(st.ep_cnt.data(), d.ep_cnt, sizeof(int) * g.pins);
  back(st.marker.data(), d.marker, sizeof(int) * K);
  back(st.send.data(), d.send, sizeof(int) * K);
  back(st.recv.data(), d.recv, sizeof(int) * K);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_status(e);
}

int fp_initial_partition(fp_instance* in) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    in->has_state = false;
    in->last_stream_dev = false;
    // auto: the device stream where it is faster than the host's (TV, MSV,
    // MSRV; CN's stream cuts its windows at most positions, whose fallback
    // part moves with every placement)
    const int m = in->pb.metric;
    const bool dev = in->stream_mode == 2 ||
                     (in->stream_mode == 0 && (m == FP_METRIC_TV || m == FP_METRIC_MSV || m == FP_METRIC_MSRV));
    if (in->stream_dev && dev) {
      const int rc = device_stream(in);
      if (rc) return rc;
      in->last_stream_dev = true;
      in->has_state = true;
      return FP_OK;
    }
    int rc = initial_partition(in->pb, in->st);
    if (rc) return rc;
    cudaSetDevice(in->ctx->device);
    rc = upload_state(in);
    if (rc) return rc;
    in->has_state = true;
    return FP_OK;
  });
}

int fp_set_stream_walk(fp_instance* in, int32_t walk) {
  return fp::guarded([&]() -> int {
    if (!in || walk < 0 || walk > 1) return FP_ERR_INVALID;
    in->sa.walk = walk;
    return FP_OK;
  });
}

int fp_set_stream_mode(fp_instance* in, int32_t mode, int32_t* last_on_device) {
  return fp::guarded([&]() -> int {
    if (!in || mode < -1 || mode > 2) return FP_ERR_INVALID;
    if (mode >= 0) in->stream_mode = mode;
    if (last_on_device) *last_on_device = in->last_stream_dev ? 1 : 0;
    return FP_OK;
  });
}

int fp_reset_state(fp_instance* in) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    cudaSetDevice(in->ctx->device);
    return upload_state(in);
  });
}

int fp_refine(fp_instance* in, int32_t passes) {
  return fp::guarded([&]() -> int {
    if (!in || passes < 0 || passes > kMaxPasses) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    if (passes == 0) { in->last_passes = 0; in->last_launches = 0; return FP_OK; }
    cudaSetDevice(in->ctx->device);
    cudaStream_t s = in->ctx->stream;
    cudaError_t e = cudaMemsetAsync(in->d.moves, 0, sizeof(long long) * passes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(in->d.status, 0, sizeof(int), s);
    const bool spec =
        in->engine == FP_ENGINE_AUTO &&
        spec_supported(in->pb.metric, in->pb.K, in->ctx->max_smem, in->g.nov, in->g.noe);
    in->d.recs = spec ? in->recs : nullptr;
    in->recs_valid = false;
    if (spec) {
      static const int none[8] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff,
                                  0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
      if (e == cudaSuccess) e = cudaMemcpyAsync(in->sb.ctl, none, sizeof(none), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(in->sb.bar, 0, sizeof(unsigned) * 4, s);
      if (e == cudaSuccess && (in->fault_leave_at || in->fault_poll_limit)) {
        const unsigned hooks[4] = {0u, in->fault_leave_at, 0u, in->fault_poll_limit};
        e = cudaMemcpyAsync(in->sb.bar, hooks, sizeof(hooks), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // `hooks` is on this stack frame
      }
      if (e == cudaSuccess) e = cudaMemsetAsync(in->sb.stats, 0, sizeof(unsigned long long) * kNumStats, s);
      if (e == cudaSuccess) e = clear_spec_scratch(in->sb, in->g.noe, in->pb.K, s);
      if (e == cudaSuccess) {
        if (in->pb.metric == FP_METRIC_CN) {
          e = cudaMemsetAsync(in->sb.claim64, 0, sizeof(unsigned long long) * std::max(in->g.noe, 1), s);
          if (e == cudaSuccess) e = cudaMemsetAsync(in->sb.cn_kcnt, 0, sizeof(int) * std::max(in->g.noe, 1), s);
          if (e == cudaSuccess) e = cudaMemsetAsync(in->sb.cn_cnt, 0, sizeof(int) * 4, s);
          if (e == cudaSuccess) e = launch_spec_cn(in->d, in->sb, passes, in->ctx->num_sms, s, &in->last_grid);
        } else if (in->pb.metric == FP_METRIC_TM || in->pb.metric == FP_METRIC_MSM) {
          e = launch_spec_msg(in->d, in->sb, passes, in->ctx->num_sms, s, &in->last_grid);
        } else {
          e = launch_spec_ldg(in->d, in->sb, passes, in->ctx->num_sms, s, &in->last_grid);
        }
      }
    } else if (e == cudaSuccess) {
      e = launch_refine(in->d, passes, s);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(in->h_status, in->d.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(in->h_moves, in->d.moves, sizeof(long long) * passes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    in->last_passes = passes;
    in->last_launches = 1;
    in->recs_valid = in->d.recs != nullptr && *in->h_status == FP_OK;
    return *in->h_status;
  });
}

int fp_set_window(fp_instance* in, int32_t min_len, int32_t grow) {
  return fp::guarded([&]() -> int {
    if (!in || min_len < 0 || grow < 1) return FP_ERR_INVALID;
    in->sb.wmin = std::min(min_len, in->sb.wmax);
    in->sb.wgrow = grow;
    return FP_OK;
  });
}

int fp_set_classes(fp_instance* in, int64_t light_work, int64_t super_work) {
  return fp::guarded([&]() -> int {
    if (!in || light_work < 0 || super_work < light_work) return FP_ERR_INVALID;
    cudaSetDevice(in->ctx->device);
    return classify(in, light_work, super_work);
  });
}

static int d2h(fp_instance* in, void* dst, const void* src, size_t bytes);

int fp_set_decision_log(fp_instance* in, int32_t on) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    cudaSetDevice(in->ctx->device);
    const size_t n = (size_t)std::max(in->pb.metric == FP_METRIC_CN ? in->g.noe : in->g.nov, 1);
    in->recs_valid = false;
    if (!on) {
      if (in->recs) {
        cudaError_t e = cudaStreamSynchronize(in->ctx->stream);
        if (e == cudaSuccess) e = cudaFree(in->recs);
        in->recs = nullptr;
        in->dev_bytes -= (long long)(n * sizeof(int4));
        if (e != cudaSuccess) return cuda_status(e);
      }
      return FP_OK;
    }
    if (in->recs) return FP_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(int4));
    if (e != cudaSuccess) return cuda_status(e);
    in->recs = static_cast<int4*>(p);
    in->dev_bytes += (long long)(n * sizeof(int4));
    return FP_OK;
  });
}

int fp_get_decisions(fp_instance* in, int32_t* dest, int32_t* gain, int32_t* loss, int32_t* moved) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    if (!in->recs) return FP_ERR_STATE;
    if (!in->recs_valid) return in->last_passes > 0 && !in->d.recs ? FP_ERR_UNSUPPORTED : FP_ERR_STATE;
    const size_t n = (size_t)(in->pb.metric == FP_METRIC_CN ? in->g.noe : in->g.nov);
    std::vector<int4> h(n);
    int rc = d2h(in, h.data(), in->recs, n * sizeof(int4));
    if (rc) return rc;
    for (size_t i = 0; i < n; i++) {
      if (dest) dest[i] = h[i].x;
      if (gain) gain[i] = h[i].y;
      if (loss) loss[i] = h[i].z;
      if (moved) moved[i] = h[i].w;
    }
    return FP_OK;
  });
}

int fp_debug_barrier_fault(fp_instance* in, int32_t leave_at, int32_t poll_limit) {
  return fp::guarded([&]() -> int {
    if (!in || leave_at < 0 || poll_limit < 0) return FP_ERR_INVALID;
    in->fault_leave_at = (unsigned)leave_at;
    in->fault_poll_limit = (unsigned)poll_limit;
    return FP_OK;
  });
}

int fp_set_engine(fp_instance* in, int32_t engine) {
  return fp::guarded([&]() -> int {
    if (!in || (engine != FP_ENGINE_AUTO && engine != FP_ENGINE_SEQUENTIAL)) return FP_ERR_INVALID;
    in->engine = engine;
    return FP_OK;
  });
}

int fp_metrics(fp_instance* in, int64_t out[6]) {
  return fp::guarded([&]() -> int {
    if (!in || !out) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    cudaSetDevice(in->ctx->device);
    cudaStream_t s = in->ctx->stream;
    int launches = 0;
    cudaError_t e = launch_metrics(in->d, in->metric_scratch, in->metric_out, in->ctx->num_sms, s, &launches);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(in->h_metrics, in->metric_out, sizeof(long long) * 6, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e);
    for (int i = 0; i < 6; i++) out[i] = in->h_metrics[i];
    in->last_launches = launches;
    return FP_OK;
  });
}

static int d2h(fp_instance* in, void* dst, const void* src, size_t bytes) {
  if (!bytes) return FP_OK;
  cudaSetDevice(in->ctx->device);
  cudaStream_t s = in->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_status(e);
}

int fp_get_partition(fp_instance* in, int32_t* part_vec) {
  return fp::guarded([&]() -> int {
    if (!in || !part_vec) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    return d2h(in, part_vec, in->d.part_vec, sizeof(int) * in->g.nov);
  });
}

int fp_get_lists(fp_instance* in, int32_t* ep_len, int32_t* ep_part, int32_t* ep_cnt) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    int rc = FP_OK;
    if (ep_len && (rc = d2h(in, ep_len, in->d.ep_len, sizeof(int) * in->g.noe))) return rc;
    if (ep_part && (rc = d2h(in, ep_part, in->d.ep_part, sizeof(int) * in->g.pins))) return rc;
    if (ep_cnt && (rc = d2h(in, ep_cnt, in->d.ep_cnt, sizeof(int) * in->g.pins))) return rc;
    return FP_OK;
  });
}

int fp_set_state(fp_instance* in, const fp_state* s) {
  return fp::guarded([&]() -> int {
    if (!in) return FP_ERR_INVALID;
    HostState st;
    const int rc = state_from_caller(in->g, in->pb, s, st);
    if (rc) return rc;
    cudaSetDevice(in->ctx->device);
    in->st = std::move(st);
    in->has_state = true;
    return upload_state(in);
  });
}

int fp_get_state(fp_instance* in, fp_state* s) {
  return fp::guarded([&]() -> int {
    if (!in || !s) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    const HostGraph& g = in->g;
    const int K = in->pb.K;
    const bool msg = in->pb.metric == FP_METRIC_TM || in->pb.metric == FP_METRIC_MSM;
    int rc = FP_OK;
    if (s->part_vec && (rc = d2h(in, s->part_vec, in->d.part_vec, sizeof(int) * g.nov))) return rc;
    if (s->ep_starts)
      for (int e = 0; e < g.noe; e++) s->ep_starts[e] = (int)g.nptr[e];
    if (s->ep_ends && (rc = d2h(in, s->ep_ends, in->d.ep_len, sizeof(int) * g.noe))) return rc;
    if (s->ep_parts && (rc = d2h(in, s->ep_parts, in->d.ep_part, sizeof(int) * g.pins))) return rc;
    if (s->ep_cnt && (rc = d2h(in, s->ep_cnt, in->d.ep_cnt, sizeof(int) * g.pins))) return rc;
    if (s->part_sizes && (rc = d2h(in, s->part_sizes, in->d.part_sizes, sizeof(int) * K))) return rc;
    if (s->marker && (rc = d2h(in, s->marker, in->d.marker, sizeof(int) * K))) return rc;
    if (s->send && (rc = d2h(in, s->send, in->d.send, sizeof(int) * K))) return rc;
    if (s->recv && (rc = d2h(in, s->recv, in->d.recv, sizeof(int) * K))) return rc;
    if (s->msgs && (rc = d2h(in, s->msgs, in->d.msgs, sizeof(int) * K))) return rc;
    if (s->conn) {
      if (msg) {
        if ((rc = d2h(in, s->conn, in->d.conn, sizeof(int) * (size_t)K * K))) return rc;
      } else {
        std::fill(s->conn, s->conn + (size_t)K * K, 0);
      }
    }
    return FP_OK;
  });
}

int fp_get_part_sizes(fp_instance* in, int32_t* sizes) {
  return fp::guarded([&]() -> int {
    if (!in || !sizes) return FP_ERR_INVALID;
    if (!in->has_state) return FP_ERR_STATE;
    return d2h(in, sizes, in->d.part_sizes, sizeof(int) * in->pb.K);
  });
}

int fp_get_moves(fp_instance* in, int64_t* moves, int32_t n) {
  return fp::guarded([&]() -> int {
    if (!in || !moves || n < 0) return FP_ERR_INVALID;
    for (int i = 0; i < n; i++) moves[i] = i < in->last_passes ? in->h_moves[i] : 0;
    return FP_OK;
  });
}

int fp_create_inverse(fp_ctx* ctx, int32_t nov, int32_t noe, int64_t pins, const uint32_t* row_ptr,
                      const uint32_t* col_ind, uint32_t* row_ptr_inv, uint32_t* col_ind_inv) {
  return fp::guarded([&]() -> int {
    if (!ctx) return FP_ERR_INVALID;
    return create_inverse_device(ctx->device, ctx->stream, ctx->num_sms, nov, noe, pins, row_ptr, col_ind,
                                 row_ptr_inv, col_ind_inv);
  });
}

int fp_thin_nets_device(fp_ctx* ctx, const fp_hypergraph* h, int32_t thin_mean, int32_t thin_min, fp_graph** out) {
  return fp::guarded([&]() -> int {
    if (!ctx || !h || !out) return FP_ERR_INVALID;
    *out = nullptr;
    const int rc = validate(h);
    if (rc) return rc;
    // the driver's bound: thin_mean x (pins / (noe + .0f)), in float, then double
    const double mean = h->noe > 0 ? (double)((float)h->pins / ((float)h->noe + 0.0f)) : 0.0;
    std::unique_ptr<fp_graph> gg(new (std::nothrow) fp_graph);
    if (!gg) return FP_ERR_NOMEM;
    const int r = thin_nets_device(ctx->device, ctx->stream, ctx->num_sms, h, thin_mean * mean, thin_min, gg->g);
    if (r) return r;
    *out = gg.release();
    return FP_OK;
  });
}

int fp_bfs_order_device(fp_ctx* ctx, const fp_hypergraph* h, int32_t start, int32_t* ordering, int32_t* far_out) {
  return fp::guarded([&]() -> int {
    if (!ctx || !h || !ordering) return FP_ERR_INVALID;
    const int rc = validate(h);
    if (rc) return rc;
    if (start < 0 || start >= h->nov) return FP_ERR_INVALID;
    return bfs_order_device(ctx->device, ctx->stream, ctx->num_sms, h, start, ordering, far_out);
  });
}

int fp_get_stats(fp_instance* in, int64_t* out, int32_t n) {
  return fp::guarded([&]() -> int {
    if (!in || !out || n < 0 || n > kNumStats) return FP_ERR_INVALID;
    return d2h(in, out, in->sb.stats, sizeof(int64_t) * n);
  });
}

int fp_last_launches(fp_instance* in, int64_t* launches) {
  return fp::guarded([&]() -> int {
    if (!in || !launches) return FP_ERR_INVALID;
    *launches = in->last_launches;
    return FP_OK;
  });
}

}  // extern "C"
