// Kernel instantiations for 1D lines above 8192 points, held by a cluster pair of CTAs.
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_long(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<10240>());
  out.push_back(make_kernel_set<12288>());
  out.push_back(make_kernel_set<16384>());
}
}  // namespace qsf
