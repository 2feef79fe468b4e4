// Kernel instantiations for grid sizes 3 * 2^k, 768 .. 6144.
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_r3b(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<768>());
  out.push_back(make_kernel_set<1536>());
  out.push_back(make_kernel_set<3072>());
  out.push_back(make_kernel_set<6144>());
}
}  // namespace qsf
