// Kernel instantiations for power-of-two grid sizes 256 .. 1024.
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_p2c(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<256>());
  out.push_back(make_kernel_set<512>());
  out.push_back(make_kernel_set<1024>());
}
}  // namespace qsf
