// Facet (boundary) loads: the reference's FacetAssembler
// (assemble/facet_assembler.py:130-235) for integrands g(x) * v.
//
// One thread per selected facet s (sel[s] = element * F + local facet f):
//   t_k  = sum_b Tc[f][q][k][b] X_b          (facet tangents: d(gamma_f)/dr_k . J)
//   |F|  = |t_0| (edges) or |t_0 x t_1| (faces)
//   out[s][b][h] = sum_q w[f][q] |F| g_h(q) N[f][q][b]
// over all B nodes of the cell, as the reference scatters the whole cell's
// nodes (facet_assembler.py:500-520).  g is a constant, node data
// interpolated with the facet shape values, or per-quadrature-point values the
// caller evaluated at the points this file's x_out mode returns.  FP64
// arithmetic; the caller reduces out to the nodes with a fixed-order segment
// sum.
#include "tm_common.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
namespace facet {

constexpr int kThreads = 128;
constexpr int kMaxComp = 3;

struct Scal {
  double v[kMaxComp];
};

template <int D>
TM_D double tangent_measure(const double (&t)[D - 1][D]);

template <>
TM_D double tangent_measure<2>(const double (&t)[1][2]) {
  return sqrt(t[0][0] * t[0][0] + t[0][1] * t[0][1]);
}

template <>
TM_D double tangent_measure<3>(const double (&t)[2][3]) {
  const double c0 = t[0][1] * t[1][2] - t[0][2] * t[1][1];
  const double c1 = t[0][2] * t[1][0] - t[0][0] * t[1][2];
  const double c2 = t[0][0] * t[1][1] - t[0][1] * t[1][0];
  return sqrt(c0 * c0 + c1 * c1 + c2 * c2);
}

// tab: w [F][Qf], N [F][Qf][B], Tc [F][Qf][D-1][B] (float64)
template <class T, int D, int B, int F>
__global__ void __launch_bounds__(kThreads) facet_load_kernel(
    int64_t n_sel, int Qf, const double* __restrict__ tab, const T* __restrict__ pts,
    const int32_t* __restrict__ elems, const int64_t* __restrict__ sel, int coef_kind, const T* __restrict__ coef,
    Scal scal, int H, T* __restrict__ out, T* __restrict__ x_out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_sel) return;
  const int64_t code = sel[s];
  const int64_t e = code / F;
  const int f = (int)(code - e * F);
  const double* w = tab + (int64_t)f * Qf;
  const double* Nf = tab + (int64_t)F * Qf + (int64_t)f * Qf * B;
  const double* Tf = tab + (int64_t)F * Qf * (1 + B) + (int64_t)f * Qf * (D - 1) * B;
  int32_t node[B];
  double X[B][D];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    node[b] = elems[e * B + b];
#pragma unroll
    for (int d = 0; d < D; ++d) X[b][d] = (double)pts[(int64_t)node[b] * D + d];
  }
  if (x_out) {
    for (int q = 0; q < Qf; ++q) {
      const double* N = Nf + (int64_t)q * B;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        double x = 0.0;
#pragma unroll
        for (int b = 0; b < B; ++b) x += N[b] * X[b][d];
        x_out[(s * Qf + q) * D + d] = (T)x;
      }
    }
    return;
  }
  double acc[B][kMaxComp];
#pragma unroll
  for (int b = 0; b < B; ++b)
#pragma unroll
    for (int h = 0; h < kMaxComp; ++h) acc[b][h] = 0.0;
  for (int q = 0; q < Qf; ++q) {
    const double* N = Nf + (int64_t)q * B;
    const double* Tc = Tf + (int64_t)q * (D - 1) * B;
    double t[D - 1][D];
#pragma unroll
    for (int k = 0; k < D - 1; ++k)
#pragma unroll
      for (int d = 0; d < D; ++d) {
        double v = 0.0;
#pragma unroll
        for (int b = 0; b < B; ++b) v += Tc[k * B + b] * X[b][d];
        t[k][d] = v;
      }
    const double fxw = w[q] * tangent_measure<D>(t);
    double g[kMaxComp];
#pragma unroll
    for (int h = 0; h < kMaxComp; ++h) {
      double v = 0.0;
      if (h < H) {
        if (coef_kind == TM_COEF_SCALAR) {
          v = scal.v[h];
        } else if (coef_kind == TM_COEF_POINT) {
#pragma unroll
          for (int b = 0; b < B; ++b) v += N[b] * (double)coef[(int64_t)node[b] * H + h];
        } else {
          v = (double)coef[(s * Qf + q) * H + h];
        }
      }
      g[h] = v * fxw;
    }
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int h = 0; h < kMaxComp; ++h) acc[b][h] += g[h] * N[b];
  }
#pragma unroll
  for (int b = 0; b < B; ++b)
#pragma unroll
    for (int h = 0; h < kMaxComp; ++h)
      if (h < H) out[(s * B + b) * H + h] = (T)acc[b][h];
}

template <class T>
int launch(int32_t element, int64_t n_sel, int Qf, const double* tab, const void* pts, const int32_t* el,
           const int64_t* sel, int coef_kind, const void* coef, Scal scal, int H, void* out, void* x_out,
           cudaStream_t s) {
  const int grid = (int)((n_sel + kThreads - 1) / kThreads);
  const T* P = static_cast<const T*>(pts);
  const T* C = static_cast<const T*>(coef);
  T* O = static_cast<T*>(out);
  T* Xo = static_cast<T*>(x_out);
  switch (element) {
    case TM_TRI3:
      facet_load_kernel<T, 2, 3, 3><<<grid, kThreads, 0, s>>>(n_sel, Qf, tab, P, el, sel, coef_kind, C, scal, H, O, Xo);
      break;
    case TM_TRI6:
      facet_load_kernel<T, 2, 6, 3><<<grid, kThreads, 0, s>>>(n_sel, Qf, tab, P, el, sel, coef_kind, C, scal, H, O, Xo);
      break;
    case TM_TET4:
      facet_load_kernel<T, 3, 4, 4><<<grid, kThreads, 0, s>>>(n_sel, Qf, tab, P, el, sel, coef_kind, C, scal, H, O, Xo);
      break;
    case TM_TET10:
      facet_load_kernel<T, 3, 10, 4><<<grid, kThreads, 0, s>>>(n_sel, Qf, tab, P, el, sel, coef_kind, C, scal, H, O,
                                                               Xo);
      break;
    default:
      return TM_ERR_UNSUPPORTED;
  }
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

}  // namespace facet
}  // namespace tmg

extern "C" int tm_facet_load(int32_t element, int32_t dtype, int32_t n_quad, const double* tables,
                             const void* points, const int32_t* elements, const int64_t* sel, int64_t n_sel,
                             int32_t coef_kind, const void* coef, const double* scal, int32_t n_comp, void* out,
                             void* x_out, void* stream) {
  if (n_sel < 0 || n_quad < 1 || n_quad > 16) return TM_ERR_INVALID;
  if (n_sel == 0) return TM_OK;
  if (!tables || !points || !elements || !sel) return TM_ERR_INVALID;
  if (!x_out) {
    if (!out || n_comp < 1 || n_comp > tmg::facet::kMaxComp) return TM_ERR_INVALID;
    const bool has_coef = coef_kind == TM_COEF_SCALAR
                              ? scal != nullptr
                              : (coef_kind == TM_COEF_POINT || coef_kind == TM_COEF_QUAD) && coef != nullptr;
    if (!has_coef) return TM_ERR_INVALID;
  }
  tmg::facet::Scal sv{};
  if (!x_out && coef_kind == TM_COEF_SCALAR)
    for (int h = 0; h < n_comp; ++h) sv.v[h] = scal[h];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == TM_F64)
    return tmg::facet::launch<double>(element, n_sel, n_quad, tables, points, elements, sel, coef_kind, coef, sv,
                                      n_comp, out, x_out, s);
  if (dtype == TM_F32)
    return tmg::facet::launch<float>(element, n_sel, n_quad, tables, points, elements, sel, coef_kind, coef, sv,
                                     n_comp, out, x_out, s);
  return TM_ERR_INVALID;
}
