// Device-side data of one resident instance and small block-level helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fp {

constexpr int kThreads = 512;                 // refinement CTA size
constexpr int kWarps = kThreads / 32;

// Everything the refinement kernels read or write, as device pointers.
struct DevInstance {
  int nov, noe;
  long long pins;
  int K;
  int metric;
  double C;          // (W / K) * eps_factor
  int max_pw;        // TV: (W/K) + (W/K)*0.1, truncated (TV/partition.cpp:95)
  int min_pw;        // TV: (W/K) - (W/K)*0.1, truncated (TV/partition.cpp:96)
  // hypergraph (read-only)
  const uint32_t* vptr;
  const uint32_t* vnets;
  const uint32_t* nptr;    // also the slot offset of each net's part list
  const uint32_t* npins;
  const int* src;
  const int* w;
  const int* order;
  // refinement state
  int* part_vec;
  int* ep_len;
  int* ep_part;
  int* ep_cnt;
  int* part_sizes;   // K
  int* marker;       // K (TV)
  int* send;         // K (MSV, MSRV)
  int* recv;         // K (MSRV)
  int* conn;         // K*K (TM, MSM)
  int* msgs;         // K (TM, MSM)
  uint32_t* zrow;    // K*K/32 bits: conn[k][r] == 0 (TM, MSM)
  uint32_t* zcol;    // K*K/32 bits: conn[s][k] == 0, column-major (TM, MSM)
  uint32_t* c1row;   // K*K/32 bits: conn[a][b] == 1 (TM, MSM)
  uint32_t* c1col;   // K*K/32 bits: conn[a][b] == 1, column-major (TM, MSM)
  // bookkeeping
  long long* moves;  // per pass
  int* status;       // device status word, 0 = ok
  // decision records of the last pass of a refine call (fp_set_decision_log),
  // one per vertex (per net for CN): (destination, gain, loss, moved); null
  // when the log is off
  int4* recs;
};

// The device stream's inputs besides the instance and its speculation buffers
// (csrc/fp_stream.cu).
struct StreamArgs {
  const int* porder;      // vertices with nets (or all vertices), visiting order
  int npos;
  const int* iso_list;    // vertices without nets (weight 0), visiting order
  const int* iso_before;  // [npos + 1] vertices without nets before each position
  int niso;
  const int* heavy_pos;   // positions whose vertex the whole grid places, ascending
  int nheavy;
  const int* mid_pos;     // positions whose vertex one CTA evaluates, ascending
  int nmid;
  const unsigned char* pclass;   // [npos] 0 a warp evaluates, 1 a CTA, 2 the grid
  int* mark_pos;          // [K] last position whose vertex saw the part, -1: none
  uint32_t* rec;          // [pins] slot of the chosen part in each (vertex, net) pair
  // message-greedy stream (TM, MSM; csrc/fp_stream_msg.cu)
  uint32_t* prow;         // [K * words] conn > 0: bit b of row a
  uint32_t* pcol;         // [K * words] conn > 0: bit a of column b
  int* rowpos;            // [2 * K] by round parity: first position that makes an entry of row a positive
  int* colpos;            // [2 * K]
  int* saved;             // [msg_wmax * K] messages each part saves, per window offset
  uint32_t* actm;         // [msg_wmax * words] source parts active on the position's nets
  uint32_t* ownm;         // [msg_wmax * words] parts listed on the nets the position is the source of
  int msg_wmax;
  int walk;               // walk the changed decisions in the window (else cut at the first)
};
constexpr int kStreamHeavy = 4096;   // nets of a vertex the whole grid places in the device stream
// List entries a position's evaluation may read (the sum of min(|e|, K) over
// its nets) from which one CTA, or the whole grid, evaluates it.
constexpr long long kStreamCtaWork = 4096;
constexpr long long kStreamGridWork = 65536;
constexpr int kStreamMaxK = 1024;    // shared memory of the device stream's CTAs
constexpr int kMsgStreamCta = 1024;  // nets of a vertex one CTA places alone in the message-greedy stream

// Round statistics kept per instance (fp_get_stats).
constexpr int kNumStats = 48;

// Whole-grid vertices one window may hold (slots of the whole-grid tallies).
constexpr int kMaxGridVerts = 8;

// Device buffers of the speculative engine (fp_spec.cu), allocated with the
// instance.
struct SpecBuf {
  unsigned* bar;         // [4] grid barrier: arrivals, generation, abort
  int* ctl;              // [8] per-round words: [2,3] first max-touching mover (by round
                         //     parity), [4,5] cut (by validation pass parity)
  int* dec;              // [wmax] (own part << 16) | decision per window offset
  unsigned char* flag;   // [wmax] bit0 mover, bit1 stale-marker risk, bit2 CTA / grid evaluated,
                         //     bit3 isolated, bit4 accepted, bit5 decision fixed exact in the
                         //     window, bit6 claims of a replaced move held (rec_slot2)
  int* dfix;             // [wmax] exact decision of a position whose size check failed
  int* slack;            // [wmax] part-size drift the decision tolerates (-1: none)
  int* vslack;           // [wmax] volume drift the accept/reject outcome tolerates
  int* wt;               // [wmax] weight moved by a mover (0 otherwise)
  int* vd;               // [wmax] largest volume change of one part by a mover
  int* rgain;            // [wmax] decision-record gain / loss of each window offset (with
  int* rloss;            //     the decision log on)
  uint32_t* scan;        // [wmax * words] parts scanned per window offset (TV)
  uint32_t* rec;         // [pins] per (vertex, net) record of a move (spec::rec_pack),
                         //     at the pair's vnets index
  const unsigned char* vclass;  // [nov] 0: warp-evaluated, 1: CTA-evaluated (medium),
                                //     2: evaluated by the whole grid
  unsigned long long* cand;  // [wmax * K] LDG candidates per window offset (part, count, first)
  int* ncand;            // [wmax]
  int4* mlist;           // [wmax] the round's movers (any order): window offset, weight,
                         //     (own part << 16) | destination
  int* midx;             // [wmax] index of a mover's mlist entry, by window offset
  int* mcnt;             // [2] their count, double-buffered by round parity
  int* wsum;             // [max_warps] per-warp sums of wt
  int* vsum;             // [max_warps] per-warp sums of vd
  unsigned long long* claim64;  // [noe] (round << 32) | ~position of the first claim (CN)
  int2* cn_moved;        // [pins] CN: (pin, window offset of its acting net) of pins to move
  int* cn_kcnt;          // [noe] CN: pins of the round's moves per net (zero between rounds)
  int2* cn_nets;         // [noe] CN: (net, packed old/new part) of the nets those moves touch
  int* cn_cnt;           // [4] CN: counts of cn_moved [0,1] and cn_nets [2,3] by round parity
  int* cn_wit;           // [nov] CN: a net of the vertex found uncut before (-1: none)
  int* claim_m;          // [noe] first mover position changing the net's part set
  int* claim_c;          // [noe] first mover position changing only counts
  uint32_t* mask_c;      // [noe] parts (mod 32) whose counts those movers change
  unsigned long long* ctab_key;  // [ctab_mask + 1] open-addressed (net << 12 | part), ~0: empty
  int* ctab_pos;         // [ctab_mask + 1] first position of a count-only mover with that (net, part)
  int* ctab_cnt;         // [ctab_mask + 1] count-only movers of the round on that (net, part)
  uint2* rec_slot;       // [pins] table slots of a count-only move's (net, own) and (net, new part)
  uint2* rec_slot2;      // [pins] (MSV / MSRV) those of a move replaced by an in-window fix
  int* ctab_over;        // [2] a probe ran past its bound this round (by round parity)
  unsigned ctab_mask;
  const int* heavy_pos;  // positions (visiting order, ascending) of vertices evaluated by
  int nheavy;            //     the whole grid (CN: nets with more than cn_grid pins)
  const int* mid_pos;    // positions (ascending) of medium vertices, evaluated by one CTA
  int nmid;              //     (CN: nets with more than cn_big pins, up to cn_grid)
  int cn_big, cn_grid;   // CN: nets with more than cn_grid pins are evaluated by the grid
                         //     (heavy_pos)
  int* hcnt;             // [2 * kMaxGridVerts * K] whole-grid vertex tallies, by round parity
  unsigned long long* hfirst;  //     and slot (the TM / MSM engine uses slot 0)
  int* hgain;            // [2 * kMaxGridVerts * K]
  int* hloss;            // [2 * kMaxGridVerts * K]
  int* hadelta;          // [2 * kMaxGridVerts * K]
  int* hmisc;            // [2 * kMaxGridVerts * 8]
  unsigned long long* mlast;  // [K] TV: (window stamp << 32) | last position whose scan holds the part
  int gmax;              // whole-grid vertices one window may hold (1 .. kMaxGridVerts)
  int wgrow;             // LDG window after a cut: this many times the last valid length,
  int wmin;              //   at least this many positions
  int maxfix;            // in-window decision fixes per window (MSV / MSRV)
  // LDG engine positions: the vertices walked in windows, in visiting order.
  // When every vertex without nets weighs 0 they are left out of the
  // positions (porder holds the others) and decided after each window:
  // iso_list holds them in visiting order, iso_before[j] counts those before
  // position j (iso_before[npos] = niso).  Otherwise porder is the visiting
  // order and niso = 0.
  const int* porder;
  int npos;
  const int* iso_list;
  const int* iso_before;
  int niso;
  unsigned long long* stats;  // [kNumStats] round statistics (see fp_get_stats)
  int wmax;              // longest window of the LDG and CN engines
  int wmax_msg;          // longest window of the TM / MSM engine (dec only)
  int max_warps;
};

// Status values a kernel can report (mirrors FP_ERR_* of the public header).
constexpr int kDevErrInvalid = -1;
constexpr int kDevErrUnsupported = -5;

__device__ __forceinline__ void dev_fail(int* status, int code) { atomicCAS(status, 0, code); }

// LDG penalty: 1 - size / C, then score * penalty, with no contraction, exactly
// the reference's double arithmetic (TV/partition.cpp:103-104).
__device__ __forceinline__ double ldg_score(int count, int size, double C) {
  double pen = __dsub_rn(1.0, __ddiv_rn((double)size, C));
  return __dmul_rn((double)count, pen);
}

// Candidate key of the LDG argmax: higher score, then smaller part, then the
// part seen first (the reference keeps the first of equal candidates).
struct LdgKey {
  double score;      // <= 0 means "not a candidate"
  int size;
  int part;
  unsigned long long first;
};

__device__ __forceinline__ bool ldg_better(const LdgKey& a, const LdgKey& b) {
  if (a.score <= 0) return false;
  if (b.score <= 0) return true;
  if (a.score != b.score) return a.score > b.score;
  if (a.size != b.size) return a.size < b.size;
  return a.first < b.first;
}

__device__ __forceinline__ LdgKey shfl_key(const LdgKey& k, int off) {
  LdgKey o;
  o.score = __shfl_xor_sync(0xffffffffu, k.score, off);
  o.size = __shfl_xor_sync(0xffffffffu, k.size, off);
  o.part = __shfl_xor_sync(0xffffffffu, k.part, off);
  o.first = __shfl_xor_sync(0xffffffffu, k.first, off);
  return o;
}

// Block-wide LDG argmax; every thread gets the winner (part = -1 if none).
// scratch holds one entry per warp of the launched block.
__device__ __forceinline__ LdgKey block_ldg_argmax(LdgKey k, LdgKey* scratch) {
  for (int off = 16; off; off >>= 1) {
    LdgKey o = shfl_key(k, off);
    if (ldg_better(o, k)) k = o;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[warp] = k;
  __syncthreads();
  if (warp == 0) {
    k = lane < (int)(blockDim.x >> 5) ? scratch[lane] : LdgKey{-1.0, 0, -1, ~0ull};
    for (int off = 16; off; off >>= 1) {
      LdgKey o = shfl_key(k, off);
      if (ldg_better(o, k)) k = o;
    }
    if (lane == 0) scratch[0] = k;
  }
  __syncthreads();
  k = scratch[0];
  __syncthreads();
  return k;
}

// Block-wide minimum of a 64-bit key (scratch: one entry per warp of the block).
__device__ __forceinline__ unsigned long long block_min_u64(unsigned long long x, unsigned long long* scratch) {
  for (int off = 16; off; off >>= 1) {
    unsigned long long o = __shfl_xor_sync(0xffffffffu, x, off);
    x = o < x ? o : x;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[warp] = x;
  __syncthreads();
  if (warp == 0) {
    x = lane < (int)(blockDim.x >> 5) ? scratch[lane] : ~0ull;
    for (int off = 16; off; off >>= 1) {
      unsigned long long o = __shfl_xor_sync(0xffffffffu, x, off);
      x = o < x ? o : x;
    }
    if (lane == 0) scratch[0] = x;
  }
  __syncthreads();
  x = scratch[0];
  __syncthreads();
  return x;
}

// Least-loaded part, lowest index on ties (TV/partition.cpp:118-132).
__device__ __forceinline__ int block_min_loaded(const int* sizes, int K, unsigned long long* scratch) {
  unsigned long long best = ~0ull;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    // sizes are non-negative; bias keeps signed order if one ever is not.
    unsigned long long key = ((unsigned long long)((unsigned)sizes[p] ^ 0x80000000u) << 32) | (unsigned)p;
    best = key < best ? key : best;
  }
  best = block_min_u64(best, scratch);
  return (int)(best & 0xffffffffu);
}

}  // namespace fp
