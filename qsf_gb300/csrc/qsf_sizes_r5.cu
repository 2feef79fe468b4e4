// Kernel instantiations for grid sizes 5 * 2^k (20 .. 5120).
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_r5(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<20>());
  out.push_back(make_kernel_set<40>());
  out.push_back(make_kernel_set<80>());
  out.push_back(make_kernel_set<160>());
  out.push_back(make_kernel_set<320>());
  out.push_back(make_kernel_set<640>());
  out.push_back(make_kernel_set<1280>());
  out.push_back(make_kernel_set<2560>());
  out.push_back(make_kernel_set<5120>());
}
}  // namespace qsf
