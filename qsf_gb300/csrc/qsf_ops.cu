// qsf_ops.cu -- granular members of the reference's LocalGrid beyond the split step:
// average_der<X, dir, PotentialEnergy> (grid.h:443-465), the expectation value of the
// potential's central difference along one axis (the dipole-acceleration form of HHG
// spectra), and operation<M, R, AntiSymmetrize<2|3>> (grid.h:611-723), the exchange
// antisymmetrisation of two or three electrons' coordinates.
#include <string>

#include "qsf_internal.h"

using namespace qsf;

namespace {

int ops_blocks(long long m) {
  long long b = (m + 255) / 256;
  return (int)std::min<long long>(std::max<long long>(b, 1), (long long)device_sm_count() * 8);
}

// per-block sums of |psi|^2 (V(x + dx e_dir) - V(x - dx e_dir)); the shifted positions
// one node past either edge come from the same linear formula (coords.h:132-135)
__global__ void __launch_bounds__(256) k_average_der(GridDev g, int dir, double* partials) {
  __shared__ double red[32];
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.m; p += stride) {
    int idx[kMaxDim];
    double cp[kMaxDim], cm[kMaxDim];
    unflatten(g, p, idx);
    for (int d = 0; d < g.dim; ++d) {
      cp[d] = g.ax[d].xmin + (double)(idx[d] + (d == dir ? 1 : 0)) * g.ax[d].dx;
      cm[d] = g.ax[d].xmin + (double)(idx[d] - (d == dir ? 1 : 0)) * g.ax[d].dx;
    }
    const double2 v = g.psi[p];
    acc += (v.x * v.x + v.y * v.y) * (potential_at(g, cp) - potential_at(g, cm));
  }
  block_sum<1>(&acc, red);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__device__ __forceinline__ double2 csub2(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }

// two particles, dim 2: psi(i, j) -= psi(j, i) with the values before the operation;
// each unordered pair is updated by one thread
__global__ void k_antisym2_2d(GridDev g) {
  const long long n = g.ax[0].n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.m; t += stride) {
    const long long i = t / n, j = t % n;
    if (i > j) continue;
    const double2 a = g.psi[i * n + j], b = g.psi[j * n + i];
    g.psi[i * n + j] = csub2(a, b);
    if (i != j) g.psi[j * n + i] = csub2(b, a);
  }
}

// two particles, dim 3 (axes 1 and 2): for k < j psi(i,j,k) -= psi(i,k,j) and
// psi(i,k,j) = -psi(i,j,k); psi(i,j,j) = 0
__global__ void k_antisym2_3d(GridDev g) {
  const long long n = g.ax[0].n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.m; t += stride) {
    const long long i = t / (n * n), j = (t / n) % n, k = t % n;
    if (k > j) continue;
    if (k == j) {
      g.psi[t] = make_double2(0.0, 0.0);
      continue;
    }
    const long long s = (i * n + k) * n + j;
    const double2 v = csub2(g.psi[t], g.psi[s]);
    g.psi[t] = v;
    g.psi[s] = cneg(v);
  }
}

// three particles, dim 3: for i > j > k the even permutations of (i,j,k) get
// psi(i,j,k) + [psi(j,k,i) + psi(k,i,j) - psi(j,i,k) - psi(i,k,j) - psi(k,j,i)] (that
// order of additions), the odd ones its negative; points with two equal indices -> 0
__global__ void k_antisym3_3d(GridDev g) {
  const long long n = g.ax[0].n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < g.m; t += stride) {
    const long long i = t / (n * n), j = (t / n) % n, k = t % n;
    if (i == j || j == k || i == k) {
      g.psi[t] = make_double2(0.0, 0.0);
      continue;
    }
    if (!(i > j && j > k)) continue;
    auto at = [&](long long a, long long b, long long c) { return (a * n + b) * n + c; };
    const double2 r2 = g.psi[at(j, k, i)], r3 = g.psi[at(k, i, j)];
    const double2 s1 = g.psi[at(j, i, k)], s2 = g.psi[at(i, k, j)], s3 = g.psi[at(k, j, i)];
    const double2 sum = make_double2(r2.x + r3.x - s1.x - s2.x - s3.x, r2.y + r3.y - s1.y - s2.y - s3.y);
    const double2 v0 = g.psi[t];
    const double2 v = make_double2(v0.x + sum.x, v0.y + sum.y);
    g.psi[t] = v;
    g.psi[at(j, k, i)] = v;
    g.psi[at(k, i, j)] = v;
    g.psi[at(j, i, k)] = cneg(v);
    g.psi[at(i, k, j)] = cneg(v);
    g.psi[at(k, j, i)] = cneg(v);
  }
}

}  // namespace

extern "C" {

int qsf_average_der(qsf_grid* g, int dir, double* out) {
  if (!g || !out || dir < 0 || dir >= g->G.dim) return fail(QSF_EINVAL, "qsf_average_der: bad argument");
  const GridDev& G = g->G;
  const int nb = std::min(256, ops_blocks(G.m));
  double* part = nullptr;
  int rc = dev_alloc(part, (size_t)nb);
  if (rc) return rc;
  std::vector<double> h((size_t)nb);
  k_average_der<<<nb, 256, 0, g->stream>>>(G, dir, part);
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, g->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(g->stream);
  cudaFree(part);
  if (ce != cudaSuccess) return fail(QSF_ECUDA, std::string("average_der: ") + cudaGetErrorString(ce));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s * G.dV * G.ax[dir].inv_2dx;
  return QSF_OK;
}

int qsf_antisymmetrize(qsf_grid* g, int particles) {
  if (!g || (particles != 2 && particles != 3)) return fail(QSF_EINVAL, "qsf_antisymmetrize: bad argument");
  const GridDev& G = g->G;
  if (G.dim >= 2) {
    for (int d = 1; d < G.dim; ++d)
      if (G.ax[d].n != G.ax[0].n) return fail(QSF_EINVAL, "qsf_antisymmetrize: axes of different lengths");
  }
  const int nb = ops_blocks(G.m);
  if (particles == 2 && G.dim == 2) k_antisym2_2d<<<nb, 256, 0, g->stream>>>(G);
  else if (particles == 2 && G.dim == 3) k_antisym2_3d<<<nb, 256, 0, g->stream>>>(G);
  else if (particles == 3 && G.dim == 3) k_antisym3_3d<<<nb, 256, 0, g->stream>>>(G);
  // other combinations leave psi unchanged, as the reference does
  QSF_CU(cudaGetLastError());
  return QSF_OK;
}

}  // extern "C"
