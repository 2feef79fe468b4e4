// Kernel instantiations for grid sizes 3 * 2^k, 12 .. 384 (the rest in qsf_sizes_r3b.cu).
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_r3b(std::vector<KernelSet>& out);
void add_sizes_r3(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<12>());
  out.push_back(make_kernel_set<24>());
  out.push_back(make_kernel_set<48>());
  out.push_back(make_kernel_set<96>());
  out.push_back(make_kernel_set<192>());
  out.push_back(make_kernel_set<384>());
  add_sizes_r3b(out);
}
}  // namespace qsf
