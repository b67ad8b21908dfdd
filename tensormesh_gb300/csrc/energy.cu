// Neo-Hookean hyperelastic energy and its displacement gradient (the
// reference's NeoHookeanModel.energy, assemble/builtin.py:220-334, and the
// autograd of ElementAssembler.energy, element_assembler.py:468-680).
//
// One thread per element, FP64 arithmetic (one log per quadrature point):
//   J_x[i][j] = sum_b dN_b/dxi_i X_b[j], grad N_b = J_x^-1 row contraction,
//   F = I + sum_b u_b (x) grad N_b, psi = mu/2 (|F|^2 - d) - mu ln J + lam/2 ln^2 J,
//   energy_e = sum_q w_q |det J_x| psi,
//   g_e[b][i] = sum_q w_q |det J_x| sum_j P[i][j] grad N_b[j],
//   P = mu F + (lam ln J - mu) F^-T.
// The per-element energies and per-(element, node) gradients are reduced by
// the caller in a fixed order (a deterministic sum and a sorted segment sum).
#include "tm_common.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
namespace nh {

template <int D> struct Mat;
template <> struct Mat<2> {
  static TM_D double det(const double (&a)[2][2]) { return a[0][0] * a[1][1] - a[0][1] * a[1][0]; }
  static TM_D void inv(const double (&a)[2][2], double d, double (&r)[2][2]) {
    const double s = 1.0 / d;
    r[0][0] = a[1][1] * s;
    r[0][1] = -a[0][1] * s;
    r[1][0] = -a[1][0] * s;
    r[1][1] = a[0][0] * s;
  }
};
template <> struct Mat<3> {
  static TM_D double det(const double (&a)[3][3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
           a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
  }
  static TM_D void inv(const double (&a)[3][3], double d, double (&r)[3][3]) {
    const double s = 1.0 / d;
    r[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) * s;
    r[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * s;
    r[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * s;
    r[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * s;
    r[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * s;
    r[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * s;
    r[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) * s;
    r[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * s;
    r[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * s;
  }
};

template <class T, int D, int B>
__global__ void __launch_bounds__(128) neohookean_kernel(int64_t n_el, int Q, const double* __restrict__ tab,
                                                         const T* __restrict__ pts, const int32_t* __restrict__ elems,
                                                         const T* __restrict__ u, double mu, double lam,
                                                         double* __restrict__ e_out, T* __restrict__ g_out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n_el) return;
  double X[B][D], U[B][D], G[B][D];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int64_t v = elems[e * B + b];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      X[b][d] = (double)pts[v * D + d];
      U[b][d] = (double)u[v * D + d];
      G[b][d] = 0.0;
    }
  }
  double en = 0.0;
  for (int q = 0; q < Q; ++q) {
    const double* dN = tab + Q + Q * B + (int64_t)q * B * D;  // [B][D] reference gradients
    double J[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < B; ++b) s += dN[b * D + i] * X[b][j];
        J[i][j] = s;
      }
    const double dJ = Mat<D>::det(J);
    double Ji[D][D];
    Mat<D>::inv(J, dJ, Ji);
    const double jxw = tab[q] * fabs(dJ);
    double gN[B][D];
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < D; ++i) s += dN[b * D + i] * Ji[j][i];
        gN[b][j] = s;
      }
    double F[D][D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double s = i == j ? 1.0 : 0.0;
#pragma unroll
        for (int b = 0; b < B; ++b) s += U[b][i] * gN[b][j];
        F[i][j] = s;
      }
    const double dF = Mat<D>::det(F);
    const double lnJ = log(dF);
    double I1 = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) I1 += F[i][j] * F[i][j];
    en += jxw * (0.5 * mu * (I1 - D) - mu * lnJ + 0.5 * lam * lnJ * lnJ);
    if (g_out) {
      double Fi[D][D];
      Mat<D>::inv(F, dF, Fi);
      const double c = lam * lnJ - mu;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          const double P = mu * F[i][j] + c * Fi[j][i];
#pragma unroll
          for (int b = 0; b < B; ++b) G[b][i] += jxw * P * gN[b][j];
        }
    }
  }
  e_out[e] = en;
  if (g_out) {
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int d = 0; d < D; ++d) g_out[(e * B + b) * D + d] = (T)G[b][d];
  }
}

template <class T>
int launch(int32_t element, int64_t n_el, int Q, const double* tab, const void* pts, const int32_t* el, const void* u,
           double mu, double lam, double* e_out, void* g_out, cudaStream_t s) {
  const int grid = (int)((n_el + 127) / 128);
  const T* P = static_cast<const T*>(pts);
  const T* Uu = static_cast<const T*>(u);
  T* G = static_cast<T*>(g_out);
  switch (element) {
    case TM_TRI3: neohookean_kernel<T, 2, 3><<<grid, 128, 0, s>>>(n_el, Q, tab, P, el, Uu, mu, lam, e_out, G); break;
    case TM_TRI6: neohookean_kernel<T, 2, 6><<<grid, 128, 0, s>>>(n_el, Q, tab, P, el, Uu, mu, lam, e_out, G); break;
    case TM_TET4: neohookean_kernel<T, 3, 4><<<grid, 128, 0, s>>>(n_el, Q, tab, P, el, Uu, mu, lam, e_out, G); break;
    case TM_TET10: neohookean_kernel<T, 3, 10><<<grid, 128, 0, s>>>(n_el, Q, tab, P, el, Uu, mu, lam, e_out, G); break;
    default: return TM_ERR_UNSUPPORTED;
  }
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

}  // namespace nh
}  // namespace tmg

extern "C" int tm_neohookean(int32_t element, int32_t dtype, int32_t n_quad, const double* tables,
                             const void* points, const int32_t* elements, int64_t n_elements, const void* u,
                             double mu, double lam, double* energy_el, void* grad_el, void* stream) {
  if (n_elements < 0 || n_quad < 1 || n_quad > 11) return TM_ERR_INVALID;
  if (n_elements == 0) return TM_OK;
  if (!tables || !points || !elements || !u || !energy_el) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == TM_F64)
    return tmg::nh::launch<double>(element, n_elements, n_quad, tables, points, elements, u, mu, lam, energy_el,
                                   grad_el, s);
  if (dtype == TM_F32)
    return tmg::nh::launch<float>(element, n_elements, n_quad, tables, points, elements, u, mu, lam, energy_el,
                                  grad_el, s);
  return TM_ERR_INVALID;
}
