// Adjoint support: the potential gradient of one slice from the adjoint of
// its slice matrix.
//
// The slice matrix is X_n = A_n - V_n - B Gss B with the projection
// V_n[a][c] = sum_j U_nj chi_a(y_j) chi_c(y_j) (src/waveguide.f90:377-380).
// For a real loss L with Xbar = dL/dX* (so dL = 2 Re Tr(Xbar^H dX)):
//   dL/dU_nj = -2 sum_{a,c} Re(Xbar[a][c]) chi_a(y_j) chi_c(y_j)
//            = -2 sum_d kappa[d] cos(pi d y_j) / ny,
//   kappa[d] = sum_{|a-c| = d} Re Xbar[a][c] - sum_{a+c+2 = d} Re Xbar[a][c],
// the transpose of the product-to-sum projection used by the sweep kernels
// (Dirichlet modes chi_m(y) = sqrt(2/ny) sin(pi m y)).
#include "rg_device.cuh"

namespace rg {
namespace {

__global__ void grad_rows_kernel(const WgDesc* wgs, const double2* __restrict__ xbar, int n, double* grad,
                                 int64_t gstride, double scale) {
  extern __shared__ double kap[];  // [2M+1]
  const int M = wgs->M, ny = wgs->ny, nd = 2 * M + 1;
  const double* costab = wgs->costab;
  const int r = blockIdx.x;
  if (r >= n) return;
  const double2* X = xbar + (int64_t)r * M * M;
  for (int d = threadIdx.x; d < nd; d += blockDim.x) {
    double s = 0.0;
    if (d < M) {
      for (int a = 0; a + d < M; ++a) {
        s += X[(int64_t)a * M + a + d].x;
        if (d > 0) s += X[(int64_t)(a + d) * M + a].x;
      }
    }
    const int lo = d - 2 - (M - 1) > 0 ? d - 2 - (M - 1) : 0;
    const int hi = d - 2 < M - 1 ? d - 2 : M - 1;
    for (int a = lo; a <= hi; ++a) s -= X[(int64_t)a * M + (d - 2 - a)].x;
    kap[d] = s;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    const double* ct = costab + (int64_t)j * nd;
    double g = 0.0;
    for (int d = 0; d < nd; ++d) g = fma(kap[d], ct[d], g);
    grad[(int64_t)r * gstride + j] = scale * g;
  }
}

}  // namespace

int launch_grad_rows(const WgDesc* d_desc, int M, const double2* xbar, int n, double* grad, int64_t gstride,
                     cudaStream_t s) {
  if (n <= 0) return RG_OK;
  grad_rows_kernel<<<n, 256, sizeof(double) * (2 * M + 1), s>>>(d_desc, xbar, n, grad, gstride, -2.0);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace rg
