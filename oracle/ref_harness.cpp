// Driver for the reference's own sequential / OpenMP partitioners -- TEST
// INFRASTRUCTURE ONLY (used to pin the oracle restatement and to time the
// reference CPU path).  Built by oracle/Makefile into oracle/_ref/ together with
// the reference's unmodified partition.cpp, metric.cpp and utils.cpp; nothing in
// the product links it.
//
// The reference drivers (TV/tv.cpp:51-97, TM/tm.cpp:65-71, CN/cn.cpp:154-284) read
// a file, choose source vertices with rand() and pass per-net sizes; this driver
// instead takes an explicit instance (vertex -> nets CSR, net -> pins CSR, source
// per net) so that the oracle and the GPU engine see exactly the same input, and
// it passes true net sizes (the TV driver passes vertex degrees there,
// TV/tv.cpp:51, which corrupts MGV_Scratch's inverse).
//
// State capture: every reference partition() evaluates MGAV_Scratch once after
// the initial stream and once after refinement (e.g. TV/partition.cpp:276,454).
// metric.cpp is compiled with -DMGAV_Scratch=MGAV_Scratch_ref, so the call lands
// in the capturing MGAV_Scratch below, which records the part vector and the
// ordered per-net part lists and then forwards to the reference evaluator.
//
// usage: ref_<metric> <instance.fphg> <K> <passes> <threads> <capture-prefix|->
//        threads == 1 runs partition(), threads > 1 partition_par(..., threads),
//        threads == 0 partition_gpu() (TV, CN, TM, MGV, MSRV) with the
//        recording wrappers below in place of the reference's gpu_partition.cu.

#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <string>
#include <vector>
#include <chrono>
#include "partition.h"

std::chrono::duration<double, std::milli> total(0);

int MGAV_Scratch_ref(int* part_vec, unsigned int* row_ptr, unsigned int* col_ind, int* src_nodes,
                     int* ep_ends, int* ep_parts, int* ep_starts, unsigned int* net_appearence,
                     int K, int nov, int noe, int pins);

static std::string g_capture_prefix;
static int g_capture_index = 0;
static std::vector<int> g_net_start;   // true net offsets, noe + 1

int MGAV_Scratch(int* part_vec, unsigned int* row_ptr, unsigned int* col_ind, int* src_nodes,
                 int* ep_ends, int* ep_parts, int* ep_starts, unsigned int* net_appearence,
                 int K, int nov, int noe, int pins) {
  if (!g_capture_prefix.empty() && g_capture_prefix != "-") {
    std::string path = g_capture_prefix + "." + std::to_string(g_capture_index);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (f) {
      // Layout: nov, noe, part_vec[nov], ep_ends[noe], then for every net its
      // ep_ends[e] listed parts in list order.
      std::fwrite(&nov, 4, 1, f);
      std::fwrite(&noe, 4, 1, f);
      std::fwrite(part_vec, 4, nov, f);
      std::fwrite(ep_ends, 4, noe, f);
      for (int e = 0; e < noe; e++) std::fwrite(ep_parts + g_net_start[e], 4, ep_ends[e], f);
      std::fclose(f);
    }
  }
  g_capture_index++;
  return MGAV_Scratch_ref(part_vec, row_ptr, col_ind, src_nodes, ep_ends, ep_parts, ep_starts,
                          net_appearence, K, nov, noe, pins);
}

// The GPU wrappers the reference partition.cpp files declare.  partition()
// and partition_par() never call them; partition_gpu() (threads == 0 below)
// does, after its initial stream, with the state arrays it would hand to the
// GPU.  These stand-ins record exactly those arrays in <capture-prefix>.wrap
// and return without refining, so that a test sees the state a drop-in shim
// receives at the boundary.
//
// .wrap layout: a sequence of records {char name[8]; int64 count; int32 data[count]}.
static void wrap_put(FILE* f, const char* name, const int* data, long long n) {
  char tag[8] = {0};
  for (int i = 0; i < 8 && name[i]; i++) tag[i] = name[i];
  std::fwrite(tag, 1, 8, f);
  std::fwrite(&n, 8, 1, f);
  if (n > 0) std::fwrite(data, 4, (size_t)n, f);
}
static FILE* wrap_open() {
  if (g_capture_prefix.empty() || g_capture_prefix == "-") return nullptr;
  return std::fopen((g_capture_prefix + ".wrap").c_str(), "wb");
}
static void wrap_common(FILE* f, int nov, int noe, long long pins, int K, int* part_vec, int* part_sizes,
                        int* ep_starts, int* ep_ends, int* ep_parts, int* ep_cnt) {
  const int dims[4] = {nov, noe, (int)pins, K};
  wrap_put(f, "dims", dims, 4);
  wrap_put(f, "part_vec", part_vec, nov);
  wrap_put(f, "psizes", part_sizes, K);
  wrap_put(f, "ep_start", ep_starts, noe);
  wrap_put(f, "ep_ends", ep_ends, noe);
  wrap_put(f, "ep_parts", ep_parts, pins);
  wrap_put(f, "ep_cnt", ep_cnt, pins);
}

#if defined(FP_REF_TV) || defined(FP_REF_MSRV)
void partition_gpu_wrapper(unsigned int*, unsigned int*, unsigned int*, int nov, int noe, long long pins, int*,
                           int*, int K, int*, int* marker, int*, int* part_sizes, int* ep_starts, int* ep_ends,
                           int* ep_parts, int* part_vec, int* ep_cnt, double*, int, double) {
  if (FILE* f = wrap_open()) {
    wrap_common(f, nov, noe, pins, K, part_vec, part_sizes, ep_starts, ep_ends, ep_parts, ep_cnt);
    wrap_put(f, "marker", marker, K);
    std::fclose(f);
  }
}
#elif defined(FP_REF_CN)
void partition_gpu_wrapper(unsigned int*, unsigned int*, unsigned int*, int nov, int noe, long long pins, int*,
                           int*, int K, int*, int, int, unsigned int*, unsigned int*, int* part_sizes,
                           int* ep_starts, int* ep_parts, int* ep_ends, int* ep_cnt, int* part_vec) {
  if (FILE* f = wrap_open()) {
    wrap_common(f, nov, noe, pins, K, part_vec, part_sizes, ep_starts, ep_ends, ep_parts, ep_cnt);
    std::fclose(f);
  }
}
#elif defined(FP_REF_TM)
static void tm_capture(int nov, int noe, long long pins, int K, int* part_vec, int* ep_starts, int* ep_parts,
                       int* ep_ends, int* ep_cnt, int** part_connections, int* part_sizes, int* part_messages) {
  if (FILE* f = wrap_open()) {
    wrap_common(f, nov, noe, pins, K, part_vec, part_sizes, ep_starts, ep_ends, ep_parts, ep_cnt);
    std::vector<int> conn((size_t)K * K);
    for (int a = 0; a < K; a++)
      for (int b = 0; b < K; b++) conn[(size_t)a * K + b] = part_connections[a][b];
    wrap_put(f, "conn", conn.data(), (long long)K * K);
    wrap_put(f, "msgs", part_messages, K);
    std::fclose(f);
  }
}
void partition_gpu_wrapper(unsigned int*, unsigned int*, unsigned int*, int nov, int noe, long long pins, int*,
                           int*, int K, int*, int, int, int* part_vec, int* ep_starts, int* ep_parts, int* ep_ends,
                           int* ep_cnt, int** part_connections, int* part_sizes, int* part_messages) {
  tm_capture(nov, noe, pins, K, part_vec, ep_starts, ep_parts, ep_ends, ep_cnt, part_connections, part_sizes,
             part_messages);
}
void partition_gpu_optimized_wrapper(unsigned int*, unsigned int*, unsigned int*, int, int, long long, int*, int*,
                                     int, int*, int, int, int*, int*, int*, int*, int*, int**, int*, int*) {
  std::abort();
}
void partition_gpu_threads_wrapper(unsigned int*, unsigned int*, unsigned int*, int, int, long long, int*, int*,
                                   int, int*, int, int, int*, int*, int*, int*, int*, int**, int*, int*) {
  std::abort();
}
#elif defined(FP_REF_MGV)
void partition_gpu_wrapper(unsigned int*, unsigned int*, unsigned int*, int nov, int noe, long long pins, int*,
                           int*, int K, int*, int, int, int* send_volumes, double*, int*, int*, int* ep_starts,
                           int* ep_parts, int* ep_ends, int* ep_cnt, int* part_sizes, int* part_vec) {
  if (FILE* f = wrap_open()) {
    wrap_common(f, nov, noe, pins, K, part_vec, part_sizes, ep_starts, ep_ends, ep_parts, ep_cnt);
    wrap_put(f, "send", send_volumes, K);
    std::fclose(f);
  }
}
#endif

template <class T>
static bool read_arr(FILE* f, std::vector<T>& v, size_t n) {
  v.resize(n);
  return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s instance.fphg K passes threads capture-prefix\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) { std::perror("open"); return 2; }
  char magic[8];
  int nov = 0, noe = 0;
  long long pins = 0;
  if (std::fread(magic, 1, 8, f) != 8 || std::fread(&nov, 4, 1, f) != 1 || std::fread(&noe, 4, 1, f) != 1 ||
      std::fread(&pins, 8, 1, f) != 1) {
    std::fprintf(stderr, "bad header\n");
    return 2;
  }
  std::vector<unsigned> vptr, vnets, nptr, npins;
  std::vector<int> src;
  if (!read_arr(f, vptr, nov + 1) || !read_arr(f, vnets, pins) || !read_arr(f, nptr, noe + 1) ||
      !read_arr(f, npins, pins) || !read_arr(f, src, noe)) {
    std::fprintf(stderr, "truncated instance\n");
    return 2;
  }
  std::fclose(f);
  int K = std::atoi(argv[2]);
  int passes = std::atoi(argv[3]);
  int threads = std::atoi(argv[4]);
  g_capture_prefix = argv[5];

  std::vector<unsigned> net_sizes(noe + 1, 0);
  for (int e = 0; e < noe; e++) net_sizes[e] = nptr[e + 1] - nptr[e];
  g_net_start.assign(nptr.begin(), nptr.end());
  std::vector<int> ordering(nov);
  for (int i = 0; i < nov; i++) ordering[i] = i;
  std::vector<int> edge_w(noe, 1);

  // The reference allocates its own state and frees nothing; buffers here are
  // owned by this process for its lifetime.
  unsigned* row_ptr = new unsigned[nov + 1];
  unsigned* col_ind = new unsigned[pins > 0 ? pins : 1];
  unsigned* col_ptr = new unsigned[noe + 1];
  unsigned* row_ind = new unsigned[pins > 0 ? pins : 1];
  unsigned* net_app = new unsigned[noe + 1];
  int* srcs = new int[noe > 0 ? noe : 1];
  int* order = new int[nov];
  int* ew = new int[noe > 0 ? noe : 1];
  for (int i = 0; i <= nov; i++) row_ptr[i] = vptr[i];
  for (long long i = 0; i < pins; i++) { col_ind[i] = vnets[i]; row_ind[i] = npins[i]; }
  for (int i = 0; i <= noe; i++) col_ptr[i] = nptr[i];
  for (int i = 0; i <= noe; i++) net_app[i] = net_sizes[i];
  for (int i = 0; i < noe; i++) { srcs[i] = src[i]; ew[i] = 1; }
  for (int i = 0; i < nov; i++) order[i] = i;

  std::string fname = g_capture_prefix.empty() || g_capture_prefix == "-" ? std::string("/tmp/fp_ref_run")
                                                                          : g_capture_prefix;
  int refi_opt = passes > 0 ? 1 : 0;
  int refi_iter = passes > 0 ? passes : 1;
#if !defined(FP_REF_MSM)
  if (threads == 0) {
#if defined(FP_REF_CN)
    partition_gpu(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter,
                  col_ptr, row_ind);
#else
    partition_gpu(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter);
#endif
    std::fflush(stdout);
    return 0;
  }
#endif
#if defined(FP_REF_CN)
  if (threads <= 1)
    partition(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter, col_ptr,
              row_ind);
  else
    partition_par(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter,
                  threads, col_ptr, row_ind);
#else
  if (threads <= 1)
    partition(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter);
  else
    partition_par(row_ptr, col_ind, net_app, nov, noe, pins, ew, srcs, K, order, fname, refi_opt, refi_iter,
                  threads);
#endif
  std::fflush(stdout);
  return 0;
}
