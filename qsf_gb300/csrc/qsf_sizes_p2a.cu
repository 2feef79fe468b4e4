// Kernel instantiations for power-of-two grid sizes 8 .. 128 (256 .. 1024 in qsf_sizes_p2c.cu).
#include <vector>
#include "qsf_kernels.cuh"
namespace qsf {
void add_sizes_p2c(std::vector<KernelSet>& out);
void add_sizes_p2a(std::vector<KernelSet>& out) {
  out.push_back(make_kernel_set<8>());
  out.push_back(make_kernel_set<16>());
  out.push_back(make_kernel_set<32>());
  out.push_back(make_kernel_set<64>());
  out.push_back(make_kernel_set<128>());
  add_sizes_p2c(out);
}
}  // namespace qsf
