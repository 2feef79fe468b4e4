// Kernel instantiations for grid sizes 5 * 2^k, 20 .. 320 (the rest in qsf_sizes_r5b.cu).
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_r5b(std::vector<KernelSet>& out);
void add_sizes_r5(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<20>());
  out.push_back(make_kernel_set<40>());
  out.push_back(make_kernel_set<80>());
  out.push_back(make_kernel_set<160>());
  out.push_back(make_kernel_set<320>());
  add_sizes_r5b(out);
}
}  // namespace qsf
