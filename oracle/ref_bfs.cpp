// Driver for the reference's BFS ordering -- TEST INFRASTRUCTURE ONLY (pins
// fp_bfs_order).  Built by oracle/Makefile into oracle/_ref/ with the
// reference's unmodified shared/utils.cpp; nothing in the product links it.
//
// Runs what the reference drivers run for -o 1 (TV/tv.cpp:110-128): the
// reference's createInverse, bfsFarthest_queue_par twice and
// bfsOrdering_queue_par, with one thread, from an explicit start vertex
// instead of rand() % nov.
//
// usage: ref_bfs <instance.fphg> <start>
// prints: farthest-first farthest-second, then the nov ordering entries.

#include <cstdio>
#include <cstdlib>
#include <vector>
#include "utils.h"

template <class T>
static bool read_arr(FILE* f, std::vector<T>& v, long long n) {
  v.resize((size_t)n);
  return n == 0 || std::fread(v.data(), sizeof(T), (size_t)n, f) == (size_t)n;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s instance.fphg start\n", argv[0]);
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
  const int start = std::atoi(argv[2]);
  std::vector<unsigned> net_app(noe + 1, 0);
  for (int e = 0; e < noe; e++) net_app[e] = nptr[e + 1] - nptr[e];
  unsigned* row_ptr_inv = nullptr;
  unsigned* col_ind_inv = nullptr;
  createInverse(vptr.data(), vnets.data(), net_app.data(), nov, noe, (int)pins, &row_ptr_inv, &col_ind_inv);
  std::vector<int> distance(nov), queue(nov), ordering(nov);
  const int f1 = bfsFarthest_queue_par(start, vptr.data(), vnets.data(), row_ptr_inv, col_ind_inv, nov,
                                       distance.data(), queue.data(), 1);
  const int f2 = bfsFarthest_queue_par(f1, vptr.data(), vnets.data(), row_ptr_inv, col_ind_inv, nov,
                                       distance.data(), queue.data(), 1);
  bfsOrdering_queue_par(f2, vptr.data(), vnets.data(), row_ptr_inv, col_ind_inv, nov, distance.data(),
                        queue.data(), ordering.data(), 1);
  std::printf("%d %d\n", f1, f2);
  for (int i = 0; i < nov; i++) std::printf("%d\n", ordering[i]);
  return 0;
}
