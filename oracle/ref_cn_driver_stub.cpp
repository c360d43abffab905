// The CN GPU wrapper that the reference's CN/partition.cpp declares; the
// reference's own CN driver (CN/cn.cpp), built into oracle/_ref/ref_cn_driver
// as TEST INFRASTRUCTURE, never calls it (no -g).  Nothing in the product
// links this file.
#include <cstdlib>

void partition_gpu_wrapper(unsigned int*, unsigned int*, unsigned int*, int, int, long long, int*, int*, int,
                           int*, int, int, unsigned int*, unsigned int*, int*, int*, int*, int*, int*, int*) {
  std::abort();
}
