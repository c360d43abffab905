/*
 * fastpart.h -- C ABI of the GB300 refinement engine for FastPartitioner.
 *
 * The library keeps one hypergraph instance resident on one GPU and runs the
 * per-metric refinement pass (CN, TV, TM, MSM, MSV, MSRV) and the six metric
 * evaluators as CUDA kernels.  Results are bit-identical to the reference's
 * single-threaded CPU refinement (`partition()` in each metric directory).
 *
 * Every function returns FP_OK (0) or a negative status; none of them prints,
 * aborts or calls exit().  Plain pointers and sizes only.
 *
 * Reference interfaces this ABI replaces (paths inside the FastPartitioner tree):
 *   partition_gpu_wrapper(...)   TV/partition.cpp:6-26, CN/partition.cpp:7-27,
 *                                TM/partition.cpp:3-7, MGV/partition.cpp:4-27,
 *                                MSRV/partition.cpp:4-25
 *   partition_gpu(...)           TV/partition.h:19, CN/partition.h:19,
 *                                TM/partition.h:16-20, MGV/partition.h:17,
 *                                MSRV/partition.h:17 (MSM has none: MSM/msm.cpp:67)
 *   metric evaluators            shared/metric.cpp:3-391
 */
#ifndef FASTPART_H
#define FASTPART_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define FP_OK                   0
#define FP_ERR_INVALID         -1  /* bad argument or malformed hypergraph            */
#define FP_ERR_CUDA            -2  /* CUDA runtime error (no device, launch failure)   */
#define FP_ERR_NOMEM           -3  /* host or device allocation failed                 */
#define FP_ERR_DEVICE_TIMEOUT  -4  /* a bounded device-side wait ran out               */
#define FP_ERR_UNSUPPORTED     -5  /* input on which the reference has undefined
                                      behaviour (e.g. a part above max_pw in the TV
                                      stream, MSRV's max-part list overflowing K)     */
#define FP_ERR_STATE           -6  /* call out of order (e.g. refine before a state)   */
#define FP_ERR_IO              -7  /* file could not be read or written                */

/* ---- metrics (the reference's directory names) ------------------------ */
#define FP_METRIC_CN    0   /* cut-net                         CN/   */
#define FP_METRIC_TV    1   /* connectivity - 1                TV/   */
#define FP_METRIC_TM    2   /* total messages                  TM/   */
#define FP_METRIC_MSM   3   /* max send messages               MSM/  */
#define FP_METRIC_MSV   4   /* max send volume                 MGV/  */
#define FP_METRIC_MSRV  5   /* max send + receive volume       MSRV/ */

/* Order of the six values returned by fp_metrics(); the order in which the
 * reference prints them (TV/partition.cpp:278-283). */
#define FP_OUT_TV   0
#define FP_OUT_CN   1
#define FP_OUT_TM   2
#define FP_OUT_MSM  3
#define FP_OUT_MSV  4
#define FP_OUT_MSRV 5

typedef struct fp_ctx fp_ctx;
typedef struct fp_instance fp_instance;
typedef struct fp_graph fp_graph;

/* A hypergraph view.  vptr/vnets: nets of each vertex in the order the
 * refinement scans them (the reference's row_ptr/col_ind).  nptr/npins: pins of
 * each net (row_ptr_inv/col_ind_inv; CN moves pins in this order).  src: the
 * source vertex of each net, which must be one of its pins (src_nodes).
 * weights: vertex weights or NULL for unit weights (the reference counts
 * vertices).  ordering: visiting order of the LDG-based metrics or NULL for
 * vertex-id order (the reference's `ordering`, -o 0). */
typedef struct {
  int32_t nov;
  int32_t noe;
  int64_t pins;
  const uint32_t* vptr;
  const uint32_t* vnets;
  const uint32_t* nptr;
  const uint32_t* npins;
  const int32_t* src;
  const int32_t* weights;
  const int32_t* ordering;
} fp_hypergraph;

/* ---- context: one GPU, one stream ------------------------------------- */
int fp_ctx_create(int32_t device, fp_ctx** out);
int fp_ctx_destroy(fp_ctx* ctx);
/* Run all subsequent work of this context on `stream` (a cudaStream_t); NULL
 * selects the context's own stream. */
int fp_ctx_set_stream(fp_ctx* ctx, void* stream);

/* Serving many requests (no counterpart in the reference, which makes one
 * call per process).
 * fp_ctx_set_arena: the context allocates `bytes` of device memory once (and
 * a few pinned host words); its instances take their buffers from it instead
 * of cudaMalloc, and releasing one frees nothing.  cudaMalloc and cudaFree
 * synchronise with the whole device, so a loop that creates and releases an
 * instance per request on one context would otherwise stall the work that
 * other contexts (other streams) have in flight.  The arena serves one
 * instance at a time: fp_instance_create returns FP_ERR_STATE while another
 * instance of the context exists, FP_ERR_NOMEM if the instance does not fit
 * (fp_instance_footprint + 64 KiB always fits: each buffer is aligned to 256
 * bytes).  bytes = 0 releases the arena; FP_ERR_STATE while an instance holds
 * it.
 * fp_ctx_set_sm_limit: the refinement and metric kernels of this context size
 * their grids for `sms` SMs (0: the whole device), so that instances of
 * several contexts, on their own streams, run on the GPU at the same time --
 * requests too small to fill the device otherwise leave most of it idle.  The
 * grid-wide engines need every CTA of a launch resident at once: the grids of
 * the contexts that run concurrently must fit the device together (their SM
 * limits summing to at most its SM count); the engine's bounded waits turn a
 * violation into FP_ERR_DEVICE_TIMEOUT, never a hang. */
int fp_ctx_set_arena(fp_ctx* ctx, int64_t bytes);
int fp_ctx_set_sm_limit(fp_ctx* ctx, int32_t sms);

/* Structural check fp_instance_create applies (no device needed): consistent
 * CSRs, distinct pins per net, non-empty nets whose source is one of their
 * pins, a permutation ordering, non-negative weights summing below 2^31. */
int fp_validate(const fp_hypergraph* hg);

/* ---- instance lifecycle ------------------------------------------------ */
/* Copies the hypergraph to the device.  eps_factor is the balance factor the
 * reference hard-codes as 1.05 (C = (nov / K) * eps, TV/partition.cpp:159-160). */
int fp_instance_create(fp_ctx* ctx, const fp_hypergraph* hg, int32_t K, int32_t metric,
                       double eps_factor, fp_instance** out);
int fp_instance_destroy(fp_instance* inst);

/* Device bytes an instance holds (the sum of its device allocations), and the
 * bytes fp_instance_create would allocate for a hypergraph of these sizes
 * (no device needed), for admission against a memory budget.  The allocator
 * rounds each allocation up, so the memory taken is a little larger.  No
 * counterpart in the reference. */
int fp_instance_device_bytes(fp_instance* inst, int64_t* bytes);
int fp_instance_footprint(int32_t nov, int32_t noe, int64_t pins, int32_t K, int32_t metric, int64_t* bytes);

/* Streaming initial partition of the metric in vertex order, kept as the
 * refinement state: part vector, per-net ordered part lists, part sizes and
 * the metric's auxiliary state (TV marker, MSV/MSRV volumes, TM/MSM K x K
 * connection counts).  Replaces the initial stream inside partition_gpu(),
 * e.g. TV/partition.cpp:1035-1092.  The TV, MSV, MSRV and CN streams can run
 * on the device when every vertex without nets weighs 0 (vertex weight =
 * degree) and K <= 1024 (fp_set_stream_mode); the other cases, and TM / MSM,
 * stream on the host and upload.  Both give the same state (the host stream's
 * result is bit for bit the reference's); the device result is copied back to
 * the host for fp_reset_state. */
int fp_initial_partition(fp_instance* inst);

/* Where fp_initial_partition streams: mode 0 (the default) on the device for
 * TV, MSV and MSRV when the instance qualifies, where it is faster than the
 * host; 1 always on the host; 2 on the device for TV, MSV, MSRV and CN
 * whenever the instance qualifies; -1 leaves the mode as it is.
 * *last_on_device (if not NULL) is set to 1 if the last fp_initial_partition
 * ran on the device.  No counterpart in the reference (its stream is CPU
 * code). */
int fp_set_stream_mode(fp_instance* inst, int32_t mode, int32_t* last_on_device);
/* Tuning of the device stream (no effect on results): walk = 1 lets a window
 * continue past the decisions that change with the exact sizes (one warp
 * takes them in order), 0 ends the window at the first.  Defaults: 1 for CN,
 * TM and MSM, 0 for TV, MSV and MSRV.  TM / MSM always walk. */
int fp_set_stream_walk(fp_instance* inst, int32_t walk);

/* Copies the host-side result of the last fp_initial_partition to the device
 * again (host -> device), discarding device-side refinement: the upload leg of
 * the reference's partition_gpu_wrapper (TV/gpu_partition.cu:366-498). */
int fp_reset_state(fp_instance* inst);

/* `passes` refinement passes on the device (REFI_ITER; the loop inside
 * partition_gpu_wrapper, TV/gpu_partition.cu:503-513).  Stream-ordered; returns
 * after the work is enqueued and its status has been read back. */
int fp_refine(fp_instance* inst, int32_t passes);

/* Refinement engine used by fp_refine: FP_ENGINE_AUTO (the speculative
 * grid-wide engine where the metric has one, else the single-CTA walk) or
 * FP_ENGINE_SEQUENTIAL (the single-CTA walk).  Both give identical results. */
#define FP_ENGINE_AUTO       0
#define FP_ENGINE_SEQUENTIAL 1
int fp_set_engine(fp_instance* inst, int32_t engine);

/* All six metrics of the current device state, in FP_OUT_* order
 * (shared/metric.cpp: TV_Refined, CN, TM_scratch, MGM_scratch, MGV_Scratch,
 * MGAV_Scratch). */
/* Tuning of the speculative engine (no effect on results).  TV / MSV / MSRV /
 * TM / MSM: a vertex whose work -- the sum over its nets of min(net size, K) --
 * is at most light_work is evaluated by one warp, at most super_work by one
 * CTA, above it by the whole grid.  Defaults: 2048 and 262144 (MSV 16384,
 * MSRV 32768, TM 65536).  CN: a net with more than light_work pins is evaluated
 * by one CTA, with more than super_work pins by the whole grid (defaults 128
 * and 1024). */
int fp_set_classes(fp_instance* inst, int64_t light_work, int64_t super_work);
/* Tuning of the speculative engine's window lengths (no effect on results;
 * TV / MSV / MSRV): after a window ends early, the next one is `grow` times
 * the committed length, at least `min_len` positions (0: one per warp of the
 * grid).  Defaults 0 and 2 (MSV) or 4 (TV, MSRV). */
int fp_set_window(fp_instance* inst, int32_t min_len, int32_t grow);
int fp_metrics(fp_instance* inst, int64_t out[6]);

/* Copies of the current device state (caller-allocated host buffers). */
int fp_get_partition(fp_instance* inst, int32_t* part_vec /* nov */);
int fp_get_lists(fp_instance* inst, int32_t* ep_len /* noe */, int32_t* ep_part /* pins */,
                 int32_t* ep_cnt /* pins */);
int fp_get_part_sizes(fp_instance* inst, int32_t* sizes /* K */);
/* Accepted moves of each of the last refine call's passes (up to n values). */
int fp_get_moves(fp_instance* inst, int64_t* moves, int32_t n);
/* ---- metric evaluation that allocates nothing ----------------------------
 * No counterpart in the reference.  For callers that must not allocate device
 * memory through this library: a serving loop that has already reserved its
 * whole device-memory budget (an extra cudaMalloc would overrun it or fail),
 * or code whose device memory belongs to another allocator (a cudaMalloc /
 * cudaFree pair beside it fragments that pool, and cudaFree waits for the
 * whole device).  It computes the six values of fp_metrics (FP_OUT_* order)
 * from a refinement state that the caller keeps in its own device memory:
 * nptr (noe + 1 net offsets, pins in total), src (noe), part_vec (nov), ep_len
 * (noe) and ep_part (pins, each net's part list at its offset), as
 * fp_get_state lays them out.  out: 6 int64 in device memory.  The work is
 * queued on `stream` (NULL: the default stream) and the call returns without
 * waiting; out is valid once the stream reaches it.
 *
 * Its scratch is one fixed array of the library's device image (147,520
 * bytes, held on every device that loads the library until the process
 * exits), so K may be at most FP_NOALLOC_MAX_K; a larger K returns
 * FP_ERR_UNSUPPORTED.  The first call on a device, with that device current,
 * looks up the array's device address; make that first call before any stream
 * capture.  Every call on a device uses the same array: calls that can overlap
 * on the GPU (different streams, no ordering between them) race and give wrong
 * values.  A state that is not consistent (a part id outside [0, K), a list
 * longer than its net, a source outside [0, nov)) makes all six outputs -1. */
#define FP_NOALLOC_MAX_K 1024
int fp_metrics_noalloc(int32_t K, int32_t nov, int32_t noe, int64_t pins, const uint32_t* nptr,
                       const int32_t* src, const int32_t* part_vec, const int32_t* ep_len,
                       const int32_t* ep_part, int64_t* out, void* stream);

/* Decision records (no counterpart in the reference's interface: its
 * refinement loops compute them and keep none).  With the log on, fp_refine
 * records the decisions of its LAST pass: one record per vertex -- per net for
 * CN -- of (dest, gain, loss, moved), each the value the reference computes
 * for it at its turn in that pass:
 *   TV    dest = the LDG decision after the max_pw / min_pw clamps; gain /
 *         loss = leave_gain / arrival_loss when dest differs from the vertex's
 *         part, else 0 / 0 (TV/partition.cpp:318-380)
 *   MSV,  dest = the LDG decision; gain / loss = the sums over all parts of
 *   MSRV  the gains[] / losses[] vectors when dest differs, else 0 / 0
 *         (MGV/partition.cpp:294-362, MSRV/partition.cpp:308-400)
 *   TM    dest = the part moved to, -1 if none; gain = the messages the move
 *         removes; loss = the messages it adds at dest, 0 if none
 *         (TM/partition.cpp:330-450)
 *   MSM   dest = the part moved to, -1 if none; gain = the sum of the gains[]
 *         vector; loss = the improvement over the max parts at dest, -1 if none
 *         (MSM/partition.cpp:388-518)
 *   CN    per net: dest = the new part of a two-part net, -1 otherwise; gain
 *         = the pins moved (0 if an uncut net vetoed the move); loss = the old
 *         part, -1 otherwise (CN/partition.cpp:262-377)
 * moved = 1 if the move was made.  The log takes 16 bytes per record of
 * device memory (counted by fp_instance_device_bytes, not by
 * fp_instance_footprint).  fp_get_decisions copies the records of the last
 * fp_refine out (NULL members skipped); FP_ERR_STATE if the log is off or no
 * refine has run with it, FP_ERR_UNSUPPORTED if that refine ran on the
 * single-CTA walk (FP_ENGINE_SEQUENTIAL, or an instance beyond the grid-wide
 * engine's limits). */
int fp_set_decision_log(fp_instance* inst, int32_t on);
int fp_get_decisions(fp_instance* inst, int32_t* dest, int32_t* gain, int32_t* loss, int32_t* moved);

/* Failure-detection test hook of the grid-wide engine (no counterpart in the
 * reference, whose wrapper exits on any CUDA error, TV/gpu_partition.cu:10-16).
 * Every grid-wide wait of the engine is bounded: a CTA that stops arriving at
 * a barrier makes the others give up after a poll limit (about a second by
 * default), and fp_refine returns FP_ERR_DEVICE_TIMEOUT with the device
 * usable.  With leave_at = n > 0 the last CTA of the next fp_refine launches
 * leaves at its n-th barrier without arriving, as a stopped CTA would;
 * poll_limit > 0 replaces the default limit (polls of the barrier word).  Both
 * zero (the default) turns the hook off.  The refined state after a timeout is
 * partial: fp_reset_state restores the initial one. */
int fp_debug_barrier_fault(fp_instance* inst, int32_t leave_at, int32_t poll_limit);

/* Statistics of the last fp_refine on the grid-wide engine (up to 48 values):
 * [0] windows, [1] whole-grid evaluations of heavy vertices (CN: nets), [2] moves
 * committed from windows, [3..8] windows ended by: nothing (fully valid), a
 * possibly stale TV marker, part-size drift, volume drift, a max-volume part
 * changing, a shared net; [9] vertices walked in windows; [16..19] nanoseconds
 * in evaluate, validate, commit phases and (TM / MSM) whole-grid decisions; TV / MSV /
 * MSRV also: [20] nanoseconds computing the round state, [21] / [23] SM cycles
 * summed over windows of the slowest warp / CTA evaluation, [25] / [26] SM
 * cycles and count of warp evaluations, [27] / [28] windows ended by an earlier
 * mover changing the count of the position's own part on a shared net / by a
 * part-set change after earlier count changes ([8] then counts part-set
 * changes only), [29..31] SM cycles of CTA evaluations in tally, decision and
 * the rest; nanoseconds summed over windows of: [32] the slowest CTA's
 * evaluation of its own positions (light and medium), [33] the whole-grid
 * vertices' decision and accept phases, [34] the slowest CTA's tally of
 * whole-grid vertex slices, [35] the slowest CTA's validation; [40] CTA
 * evaluations; [41..43] SM cycles of warp evaluations in tally, decision and
 * the rest; [44] decisions fixed inside a window (MSV / MSRV); [45..47]
 * nanoseconds summed over CTAs and validation passes in prefix sums, light
 * positions and the rest (medium and whole-grid vertices).  The per-warp and
 * per-CTA timings ([21..26], [29..43] except the [33] phase time, [45..47]) are
 * collected only by a library built with FP_TIMING_STATS defined, and are zero
 * otherwise. */
int fp_get_stats(fp_instance* inst, int64_t* out, int32_t n);
/* Number of kernel launches the last fp_refine / fp_metrics call enqueued. */
int fp_last_launches(fp_instance* inst, int64_t* launches);

const char* fp_strerror(int status);

/* ---- host hypergraphs: generator and file formats ---------------------- */
typedef struct {
  int32_t nov, noe;
  int32_t size_lo, size_hi;   /* net size range                                   */
  double size_alpha;          /* > 0: Zipf(alpha) sizes clipped to [lo, hi]         */
  double pin_beta;            /* > 0: pins by Zipf(beta) popularity, else uniform   */
  int32_t src_rule;           /* 0: lowest-id pin is the source, 1: first drawn     */
  int32_t sort_pins;          /* 1: pins of a net sorted by id                      */
  int32_t weight_rule;        /* 0: unit weights, 1: weight = degree                */
  uint64_t seed;
} fp_gen_params;

int fp_generate(const fp_gen_params* p, fp_graph** out);
/* BFS visiting order, the reference's -o 1 (TV/tv.cpp:110-128 with one thread;
 * replaces bfsFarthest_queue_par x 2 + bfsOrdering_queue_par,
 * shared/utils.cpp:433-536).  A BFS from `start` finds the farthest vertex
 * (lowest id on ties), a BFS from it the farthest again, and a BFS from that
 * one lists the vertices level by level in discovery order: a vertex's nets in
 * vertex -> nets order, a net's pins in ascending id (createInverse's order).
 * The reference driver starts from rand() % nov.  Writes nov entries to
 * `ordering` (-1 past the reached vertices) and, if far_out is not null, the
 * two farthest vertices.  FP_ERR_UNSUPPORTED if a vertex is not reached: the
 * reference's partitioners would then read ordering entries of -1.  Host code
 * (no GPU). */
int fp_bfs_order(const fp_hypergraph* h, int32_t start, int32_t* ordering, int32_t* far_out);
/* Builds a host graph from a net -> pins CSR (the .hg orientation of the TV and
 * CN drivers): vertex -> nets is its transpose, nets ascending per vertex. */
int fp_graph_from_nets(int32_t nov, int32_t noe, const uint32_t* nptr, const uint32_t* npins,
                       const int32_t* src, fp_graph** out);
/* Builds a host graph from a vertex -> nets CSR (the reference's row_ptr /
 * col_ind as partition() receives them): net -> pins is built as the
 * reference's createInverse does (shared/utils.cpp:32-56), pins ascending per
 * net.  src NULL: lowest-id pin of each net. */
int fp_graph_from_vertices(int32_t nov, int32_t noe, const uint32_t* vptr, const uint32_t* vnets,
                           const int32_t* src, fp_graph** out);
/* Reads a PaToH-like .hg file (shared/hypergraph_rw.cpp:97-242), honouring an
 * existing `<path>.plbin` cache exactly as the reference does.  `transpose` = 1
 * makes file lines nets (TV, CN drivers); 0 makes file lines vertices (TM, MSM,
 * MGV, MSRV drivers, TM/tm.cpp:65).  Sources: src_rule as in fp_gen_params,
 * applied to each net's pins. */
int fp_read_patohlike(const char* path, int32_t transpose, int32_t write_cache, fp_graph** out);
/* CN thinning (-m 1 -n thin_min -z thin_mean; replaces the driver's filter,
 * CN/cn.cpp:201-268): keeps the nets with fewer than thin_mean x (pins / noe,
 * in float) and fewer than thin_min pins, renumbered in order, with their pins
 * and sources; every vertex keeps its kept nets in its own order.  The driver
 * then runs the ordinary CN partition on the thinned hypergraph
 * (thin_partition, CN/partition.cpp:841-1196, is partition() writing into the
 * caller's part vector) and evaluates the six metrics on the full one. */
int fp_thin_nets(const fp_hypergraph* h, int32_t thin_mean, int32_t thin_min, fp_graph** out);

/* The same three hypergraph transforms on the context's GPU (csrc/fp_ingest.cu),
 * with results equal to the host forms' bit for bit:
 *
 * fp_create_inverse: the reference's createInverse (shared/utils.cpp:32-56)
 * with caller-owned host arrays -- from the vertex -> nets CSR (row_ptr[nov+1],
 * col_ind[pins]) the net -> pins CSR (row_ptr_inv[noe+1], col_ind_inv[pins]),
 * each net's pins in ascending vertex id.  The per-net counts the reference
 * takes (net_appearence) are counted on the device.  FP_ERR_INVALID if
 * row_ptr is not a CSR of `pins` entries or a net id is not below noe.
 *
 * fp_thin_nets_device: fp_thin_nets (CN/cn.cpp:201-268) on the device.
 *
 * fp_bfs_order_device: fp_bfs_order (shared/utils.cpp:433-536) on the device:
 * the same three searches, the same ordering and farthest vertices, the same
 * FP_ERR_UNSUPPORTED when a vertex is not reached. */
int fp_create_inverse(fp_ctx* ctx, int32_t nov, int32_t noe, int64_t pins, const uint32_t* row_ptr,
                      const uint32_t* col_ind, uint32_t* row_ptr_inv, uint32_t* col_ind_inv);
int fp_thin_nets_device(fp_ctx* ctx, const fp_hypergraph* h, int32_t thin_mean, int32_t thin_min, fp_graph** out);
int fp_bfs_order_device(fp_ctx* ctx, const fp_hypergraph* h, int32_t start, int32_t* ordering, int32_t* far_out);
int fp_write_patohlike(const fp_graph* g, const char* path);
int fp_graph_view(const fp_graph* g, fp_hypergraph* view);
int fp_graph_destroy(fp_graph* g);

/* ---- refinement state in the reference's layout ----------------------- */
/* The arrays the reference's partition() hands to its GPU wrapper after the
 * initial stream (partition_gpu_wrapper, TV/partition.cpp:6-26,
 * MGV/partition.cpp:4-27, MSRV/partition.cpp:4-25, TM/partition.cpp:3-7).
 * Sizes: part_vec nov; ep_starts / ep_ends noe; ep_parts / ep_cnt pins (empty
 * slots -1 / 0); part_sizes, marker, send, recv, msgs K; conn K*K row-major.
 * Net e's list is ep_parts / ep_cnt [ep_starts[e], ep_starts[e] + ep_ends[e]):
 * ep_ends[e] is lambda(e), the NUMBER of parts listed, not an end offset -- the
 * stream counts it up from 0 (TV/partition.cpp:1066-1075) and the reference's
 * metric code reads it as that count (TV(), CN(), shared/metric.cpp:3-14,57-68). */
typedef struct fp_state {
  int32_t* part_vec;
  int32_t* ep_starts;   /* must equal the net offsets (prefix of net sizes)        */
  int32_t* ep_ends;     /* lambda(e): parts listed for net e                       */
  int32_t* ep_parts;
  int32_t* ep_cnt;
  int32_t* part_sizes;  /* NULL on set: recounted from part_vec and the weights    */
  int32_t* marker;      /* TV's last scanner per part; NULL on set: all -1         */
  int32_t* send;        /* MSV / MSRV send volumes; NULL on set: recounted (other
                           metrics keep none: ignored on set, zero on get)         */
  int32_t* recv;        /* MSRV received volumes; NULL on set: recounted (ditto)   */
  int32_t* conn;        /* TM / MSM part_connections; NULL on set: recounted       */
  int32_t* msgs;        /* TM / MSM part_messages; NULL on set: recounted          */
} fp_state;

/* Replaces the instance's state with a caller-built one (checked against the
 * hypergraph: every list must equal the recount from part_vec); it becomes the
 * state fp_reset_state() restores.  Replaces the wrapper's upload of these
 * arrays before its refinement kernels. */
int fp_set_state(fp_instance* inst, const fp_state* st);
/* Copies the current device state out; NULL members are skipped.  ep_starts
 * is filled with the net offsets, ep_ends with lambda(e). */
int fp_get_state(fp_instance* inst, fp_state* st);
/* The check fp_set_state applies, on the host alone (no device): FP_OK if `st`
 * is a valid state of hypergraph h for this K and metric -- part ids in [0, K),
 * ep_starts the net offsets, every net's list (ep_ends[e] = lambda(e) entries)
 * exactly the parts of its pins with their counts, part_sizes (if given) the
 * weighted recount -- else FP_ERR_INVALID.  The reference keeps this invariant
 * and checks it in checkMe (MSM/partition.cpp:2-68). */
int fp_check_state(const fp_hypergraph* h, int32_t K, int32_t metric, double eps_factor, const fp_state* st);
/* The metric's streaming initial partition on the host (the CPU half of the
 * reference's partition_gpu(): TV/partition.cpp:207-264, CN/partition.cpp:
 * 132-221, TM/partition.cpp:87-250, MSM/partition.cpp:146-309,
 * MGV/partition.cpp:122-189, MSRV/partition.cpp:123-196), written to `out` in
 * the fp_state layout (NULL members skipped; conn zero for the metrics that
 * keep none).  The same stream fp_initial_partition runs; no GPU needed.
 * fp_set_state then hands the state to an instance. */
int fp_stream_partition(const fp_hypergraph* h, int32_t K, int32_t metric, double eps_factor, fp_state* out);

/* ---- drop-in for partition_gpu() --------------------------------------- */
/* Same arguments and the same stdout lines as the reference's partition_gpu()
 * of the given metric: initial stream, "TV : ..." metric lines, REFI_ITER
 * device refinement passes, "After Refinement ..." lines and "Refinement took".
 * row_ptr_inv / col_ind_inv may be NULL (they are rebuilt from row_ptr/col_ind;
 * CN passes them, CN/partition.h:19).  part_vec_out (nov, may be NULL) receives
 * the refined part vector; metrics_out (12, may be NULL) the six metrics before
 * and after refinement. */
int fp_partition_gpu(int32_t metric, const uint32_t* row_ptr, const uint32_t* col_ind,
                     const uint32_t* net_appearence, int32_t nov, int32_t noe, int64_t pins,
                     const int32_t* edge_wgths, const int32_t* src_nodes, int32_t K,
                     const int32_t* ordering, const char* f_name, int32_t REFI_OPT, int32_t REFI_ITER,
                     const uint32_t* row_ptr_inv, const uint32_t* col_ind_inv, int32_t* part_vec_out,
                     int64_t* metrics_out);

#ifdef __cplusplus
}
#endif

#endif /* FASTPART_H */
