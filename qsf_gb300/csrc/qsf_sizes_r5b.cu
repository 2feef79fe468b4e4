// Kernel instantiations for grid sizes 5 * 2^k, 640 .. 5120.
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_r5b(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<640>());
  out.push_back(make_kernel_set<1280>());
  out.push_back(make_kernel_set<2560>());
  out.push_back(make_kernel_set<5120>());
}
}  // namespace qsf
