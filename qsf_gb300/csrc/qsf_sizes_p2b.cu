// Kernel instantiations for power-of-two grid sizes 2048 .. 8192.
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_p2b(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<2048>());
  out.push_back(make_kernel_set<4096>());
  out.push_back(make_kernel_set<8192>());
}
}  // namespace qsf
