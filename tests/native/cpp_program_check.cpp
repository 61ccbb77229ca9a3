// A grouped-GEMM program built on the C++ side (imps_cpp::program, include/imps_gb300.hpp) and
// run on the device, checked against the same products on the host:
//   stage 1: C (3 x 4)  = A (3 x 2) B (2 x 4)
//   stage 2: D (4 x 3)  = 2 C^T I (a transposed operand and a scale)
// Exit status 0 when both agree to rounding.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

#include "../../include/imps_gb300.hpp"

using imps_cpp::plan;

int main() {
  imps_cpp::context ctx(0);
  const int m = 3, k = 2, n = 4;
  std::vector<double> A(m * k), B(k * n), I(m * m, 0.0);
  for (int i = 0; i < m * k; ++i) A[i] = 0.25 * (i + 1);
  for (int i = 0; i < k * n; ++i) B[i] = 0.5 - 0.125 * i;
  for (int i = 0; i < m; ++i) I[i + m * i] = 1.0;

  imps_cpp::program prog;
  prog.slot_nelem = {m * k, k * n, m * n, m * m, n * m};  // A, B, C, I, D
  {
    auto& s = prog.stage();
    s.push_back({2, 0, m, m, n, false, {{0, 0, m, false, 1, 0, k, false, k, 1.0}}});
  }
  {
    auto& s = prog.stage();
    s.push_back({4, 0, n, n, m, false, {{2, 0, m, true, 3, 0, m, false, m, 2.0}}});
  }
  plan p = plan::program(ctx, prog);

  std::vector<double*> dev(5);
  for (int s = 0; s < 5; ++s) {
    const size_t bytes = prog.slot_nelem[s] * sizeof(double);
    if (cudaMalloc(&dev[s], bytes) != cudaSuccess) return 2;
    const double* src = s == 0 ? A.data() : s == 1 ? B.data() : s == 3 ? I.data() : nullptr;
    if (src) cudaMemcpy(dev[s], src, bytes, cudaMemcpyHostToDevice);
    else cudaMemset(dev[s], 0, bytes);
    p.bind(s, dev[s]);
  }
  p.run();
  ctx.synchronize();
  std::vector<double> D(n * m);
  cudaMemcpy(D.data(), dev[4], D.size() * sizeof(double), cudaMemcpyDeviceToHost);
  for (double* d : dev) cudaFree(d);

  double err = 0.0;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j) {
      double c = 0.0;
      for (int t = 0; t < k; ++t) c += A[i + m * t] * B[t + k * j];
      err = std::fmax(err, std::fabs(D[j + n * i] - 2.0 * c));  // D = 2 C^T
    }
  if (err > 1e-13) {
    std::printf("cpp program check failed: max error %.3e\n", err);
    return 1;
  }
  std::printf("cpp program check ok (max error %.1e)\n", err);
  return 0;
}
