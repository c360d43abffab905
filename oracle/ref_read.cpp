// Driver for the reference's PaToH-like reader -- TEST INFRASTRUCTURE ONLY
// (pins fp_read_patohlike).  Built by oracle/Makefile into oracle/_ref/ with
// the reference's unmodified shared/hypergraph_rw.cpp; nothing in the product
// links it.
//
// Calls read_patohlike (shared/hypergraph_rw.cpp:97-242) on a file -- which
// reads <file>.plbin when it exists and writes it otherwise -- and stores what
// it returns, since the reader itself prints to stdout.
//
// usage: ref_read <file.hg> <out.bin>
// out.bin: i32 ok, u32 nov, u32 noe, i64 pins, then (if ok) col_ptr[noe + 1],
//          row_ind[pins], vertex_appearence[nov] as u32.

#include <cstdio>
#include <string>
#include "hypergraph_rw.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s file.hg out.bin\n", argv[0]);
    return 2;
  }
  unsigned int* col_ptr = nullptr;
  unsigned int* row_ind = nullptr;
  unsigned int* appear = nullptr;
  unsigned int nov = 0, noe = 0;
  long long pins = 0;
  const int ok = read_patohlike(std::string(argv[1]), &col_ptr, &row_ind, &appear, nov, noe, pins) ? 1 : 0;
  FILE* f = std::fopen(argv[2], "wb");
  if (!f) { std::perror("open"); return 2; }
  std::fwrite(&ok, 4, 1, f);
  std::fwrite(&nov, 4, 1, f);
  std::fwrite(&noe, 4, 1, f);
  std::fwrite(&pins, 8, 1, f);
  if (ok) {
    std::fwrite(col_ptr, 4, (size_t)noe + 1, f);
    std::fwrite(row_ind, 4, (size_t)pins, f);
    std::fwrite(appear, 4, nov, f);
  }
  std::fclose(f);
  return 0;
}
