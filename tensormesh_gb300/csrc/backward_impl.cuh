// Adjoint (backward) assembly: gradients of a scalar loss L with respect to
// the nodal coordinates and the integrand coefficient, given dL/d(values).
//
// The reference obtains these by autograd through its vmap/einsum chain,
// torch.inverse and the index_add_ scatter (element/element.py:
// 962-966, element/transformation.py:1289, assemble/projector.py:125).  Here
// one hand-written kernel runs the chain rule per element.  With
// P = dN J^-T (physical gradients), |det J| and the quadrature weight w,
// one quadrature point contributes L_q = w c |det J| phi(P) and
//     dL_q/dJ = A_q = w c |det J| (phi I - P^T M) J^-1,   M = d phi / d P,
//     dL/dX   = sum_q dN_q A_q^T                 (J = dN^T X),
//     dL/dc   = sum_q w |det J| phi.
// Laplace: phi = sum_ij S_ij P_i.P_j, M = (S + S^T) P.  Mass: phi = N^T S N,
// M = 0.  Elasticity: phi = sum S_{ia,jb} (lam P_ia P_jb + mu (d_ab P_i.P_j +
// P_ib P_ja)).  Load: phi = sum_ih S_ih f_h N_i.
//
// The patch structure of the forward pass is reused in reverse: the owner of
// each CSR row broadcasts dL/dK of its row into the staged element slots
// (phase B reversed); then every element of the patch computes its partial
// gradients from the rows this patch owns (phase A reversed) and writes them
// to per-(patch, element) buffers.  Each (element, row) incidence is owned by
// exactly one patch, so summing the partials of an element's patches -- in a
// fixed order, by tm_segment_sum -- gives the full gradient deterministically.
#pragma once
#include "assemble_impl.cuh"

namespace tmg {

template <int EL, int FORM, int H, class T, class R>
__global__ void __launch_bounds__(kThreads)
patch_backward_kernel(tm_patch_plan plan, tm_assemble_args args, tm_backward_args bw, int chunk) {
  using L = Layout<EL, FORM, H>;
  constexpr int D = L::D, B = L::B, SE = L::SE, HH = L::HH;
  const int p = blockIdx.x;
  const int tid = threadIdx.x;
  const int Q = args.n_quad;
  const int vbeg = plan.vptr[p], nv = plan.vptr[p + 1] - vbeg;
  const int ebeg = plan.eptr[p], ne = plan.eptr[p + 1] - ebeg;
  const int rbeg = plan.rptr[p], nr = plan.rptr[p + 1] - rbeg;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* s_w = reinterpret_cast<R*>(smem_raw);
  R* s_N = s_w + kMaxQuad;
  R* s_dN = s_N + kMaxQuad * B;
  R* s_X = s_dN + kMaxQuad * B * D;
  R* s_pc = s_X + plan.max_vtx * D;
  const int pc_len = (args.coef_kind == TM_COEF_POINT) ? plan.max_vtx * (L::kLoad ? H : 1) : 0;
  R* s_G = s_pc + pc_len;                          // staged dL/dK of owned rows [SE][chunk]
  int* s_cur = reinterpret_cast<int*>(s_G + chunk * SE);

  for (int i = tid; i < Q; i += kThreads) s_w[i] = Num<R>::from_double(args.tables[i]);
  for (int i = tid; i < Q * B; i += kThreads) s_N[i] = Num<R>::from_double(args.tables[Q + i]);
  for (int i = tid; i < Q * B * D; i += kThreads) s_dN[i] = Num<R>::from_double(args.tables[Q + Q * B + i]);
  const T* pts = static_cast<const T*>(args.points);
  for (int i = tid; i < nv * D; i += kThreads) {
    int v = plan.vtx[vbeg + i / D];
    s_X[i] = tm_load<R, T>(pts[(int64_t)v * D + i % D]);
  }
  constexpr int PC = L::kLoad ? H : 1;
  if (args.coef_kind == TM_COEF_POINT) {
    const T* pc = static_cast<const T*>(args.coef);
    for (int i = tid; i < nv * PC; i += kThreads) {
      int v = plan.vtx[vbeg + i / PC];
      s_pc[i] = tm_load<R, T>(pc[(int64_t)v * PC + i % PC]);
    }
  }
  for (int i = tid; i < nr; i += kThreads) s_cur[i] = plan.iptr[rbeg + i];
  __syncthreads();

  R scal[3];
#pragma unroll
  for (int h = 0; h < 3; ++h) scal[h] = Num<R>::from_double(args.scal[h]);
  const R lam1 = Num<R>::from_double(args.lam);
  const R mu1 = Num<R>::from_double(args.mu);
  const T* coef = static_cast<const T*>(args.coef);
  const T* G = static_cast<const T*>(bw.grad_out);
  T* out_dX = static_cast<T*>(bw.pair_dX);
  T* out_dc = static_cast<T*>(bw.pair_dcoef);

  for (int cbeg = 0; cbeg < ne; cbeg += chunk) {
    const int cend = min(ne, cbeg + chunk);
    for (int i = tid; i < chunk * SE; i += kThreads) s_G[i] = Num<R>::zero();
    __syncthreads();
    // --- phase B reversed: owned rows broadcast dL/dK into element slots ------
    for (int lr = tid; lr < nr; lr += kThreads) {
      int cur = s_cur[lr];
      const int end = plan.iptr[rbeg + lr + 1];
      const int r = plan.rows[rbeg + lr];
      const int64_t s0 = plan.indptr[r];
      const int deg = (int)(plan.indptr[r + 1] - s0);
      while (cur < end) {
        const int le = plan.inc_elem[cur];
        if (le >= cend) break;
        const int a = plan.inc_a[cur];
        const Strided<R> Gs{s_G + (le - cbeg), chunk};
        if constexpr (L::kLoad) {
#pragma unroll
          for (int h = 0; h < H; ++h) Gs[a * H + h] = tm_load<R, T>(G[(int64_t)r * H + h]);
        } else {
#pragma unroll
          for (int b = 0; b < B; ++b) {
            const int pos = plan.inc_pos[(int64_t)cur * B + b];
#pragma unroll
            for (int aa = 0; aa < H; ++aa)
#pragma unroll
              for (int bb = 0; bb < H; ++bb) {
                const int64_t slot = (int64_t)HH * s0 + (int64_t)aa * H * deg + (int64_t)pos * H + bb;
                Gs[(a * B + b) * HH + aa * H + bb] = tm_load<R, T>(G[slot]);
              }
          }
        }
        ++cur;
      }
      s_cur[lr] = cur;
    }
    __syncthreads();
    // --- phase A reversed: per-element partial gradients ---------------------
    for (int le = cbeg + tid; le < cend; le += kThreads) {
      const int pair = ebeg + le;
      const int e = plan.elem[pair];
      int lv[B];
      R X[B][D];
#pragma unroll
      for (int b = 0; b < B; ++b) {
        lv[b] = plan.econn[(int64_t)pair * B + b];
#pragma unroll
        for (int d = 0; d < D; ++d) X[b][d] = s_X[lv[b] * D + d];
      }
      const Strided<R> S{s_G + (le - cbeg), chunk};
      R ce = scal[0];
      if (args.coef_kind == TM_COEF_ELEMENT) ce = tm_load<R, T>(coef[e]);
      R dX[B][D];
#pragma unroll
      for (int b = 0; b < B; ++b)
#pragma unroll
        for (int d = 0; d < D; ++d) dX[b][d] = Num<R>::zero();
      R dce = Num<R>::zero();
      R dpc[B][PC];
#pragma unroll
      for (int b = 0; b < B; ++b)
#pragma unroll
        for (int h = 0; h < PC; ++h) dpc[b][h] = Num<R>::zero();

      for (int q = 0; q < Q; ++q) {
        const R* dNq = s_dN + q * B * D;
        const R* Nq = s_N + q * B;
        // geometry (same algebra as the forward pass) keeping J^-1 explicitly
        R J[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            R s = Num<R>::zero();
#pragma unroll
            for (int b = 0; b < B; ++b) s = s + X[b][j] * dNq[b * D + i];
            J[i][j] = s;
          }
        R adj[D][D], det;
        if constexpr (D == 2) {
          det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          adj[0][0] = J[1][1]; adj[0][1] = -J[0][1]; adj[1][0] = -J[1][0]; adj[1][1] = J[0][0];
        } else {
          adj[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
          adj[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
          adj[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
          adj[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
          adj[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
          adj[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
          adj[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
          adj[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
          adj[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
          det = J[0][0] * adj[0][0] + J[0][1] * adj[1][0] + J[0][2] * adj[2][0];
        }
        const R rdet = Num<R>::from_float(1.f) / det;
        R Jinv[D][D];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) Jinv[i][j] = adj[i][j] * rdet;
        R P[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            R s = Num<R>::zero();
#pragma unroll
            for (int i = 0; i < D; ++i) s = s + dNq[b * D + i] * Jinv[j][i];
            P[b][j] = s;
          }
        const R wdet = s_w[q] * Num<R>::abs(det);
        // coefficient at q and its source
        R cq = ce;
        if (!L::kLoad && args.coef_kind == TM_COEF_POINT) {
          R s = Num<R>::zero();
#pragma unroll
          for (int b = 0; b < B; ++b) s = s + s_pc[lv[b]] * Nq[b];
          cq = s;
        } else if (!L::kLoad && args.coef_kind == TM_COEF_QUAD) {
          cq = tm_load<R, T>(coef[(int64_t)e * Q + q]);
        }
        R phi = Num<R>::zero();
        R M[B][D];
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
          for (int d = 0; d < D; ++d) M[b][d] = Num<R>::zero();
        if constexpr (FORM == TM_FORM_LAPLACE) {
#pragma unroll
          for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) {
              const R sij = S[i * B + j];
              R dot = Num<R>::zero();
#pragma unroll
              for (int d = 0; d < D; ++d) dot = dot + P[i][d] * P[j][d];
              phi = phi + sij * dot;
#pragma unroll
              for (int d = 0; d < D; ++d) {
                M[i][d] = M[i][d] + sij * P[j][d];
                M[j][d] = M[j][d] + sij * P[i][d];
              }
            }
        } else if constexpr (FORM == TM_FORM_MASS) {
#pragma unroll
          for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) phi = phi + S[i * B + j] * (Nq[i] * Nq[j]);
        } else if constexpr (FORM == TM_FORM_ELASTICITY) {
#pragma unroll
          for (int i = 0; i < B; ++i)
#pragma unroll
            for (int j = 0; j < B; ++j) {
              const int sb = (i * B + j) * HH;
              R dot = Num<R>::zero();
#pragma unroll
              for (int d = 0; d < D; ++d) dot = dot + P[i][d] * P[j][d];
              R tr = Num<R>::zero();
#pragma unroll
              for (int a = 0; a < H; ++a) tr = tr + S[sb + a * H + a];
              phi = phi + mu1 * tr * dot;
#pragma unroll
              for (int d = 0; d < D; ++d) {
                M[i][d] = M[i][d] + mu1 * tr * P[j][d];
                M[j][d] = M[j][d] + mu1 * tr * P[i][d];
              }
#pragma unroll
              for (int a = 0; a < H; ++a)
#pragma unroll
                for (int b = 0; b < H; ++b) {
                  const R s = S[sb + a * H + b];
                  phi = phi + s * (lam1 * (P[i][a] * P[j][b]) + mu1 * (P[i][b] * P[j][a]));
                  M[i][a] = M[i][a] + lam1 * s * P[j][b];
                  M[j][b] = M[j][b] + lam1 * s * P[i][a];
                  M[i][b] = M[i][b] + mu1 * s * P[j][a];
                  M[j][a] = M[j][a] + mu1 * s * P[i][b];
                }
            }
        } else {  // load: phi = sum_ih S_ih f_h N_i ; dphi/df_h = sum_i S_ih N_i
          R fq[H], sn[H];
#pragma unroll
          for (int h = 0; h < H; ++h) {
            R s = Num<R>::zero();
#pragma unroll
            for (int i = 0; i < B; ++i) s = s + S[i * H + h] * Nq[i];
            sn[h] = s;
            if (args.coef_kind == TM_COEF_SCALAR) fq[h] = scal[h];
            else if (args.coef_kind == TM_COEF_ELEMENT) fq[h] = ce;
            else if (args.coef_kind == TM_COEF_QUAD) fq[h] = tm_load<R, T>(coef[((int64_t)e * Q + q) * H + h]);
            else {
              R t = Num<R>::zero();
#pragma unroll
              for (int b = 0; b < B; ++b) t = t + s_pc[lv[b] * H + h] * Nq[b];
              fq[h] = t;
            }
            phi = phi + sn[h] * fq[h];
          }
          if (args.coef_kind == TM_COEF_QUAD && out_dc) {
#pragma unroll
            for (int h = 0; h < H; ++h) out_dc[((int64_t)pair * Q + q) * H + h] = tm_store<T, R>(wdet * sn[h]);
          } else if (args.coef_kind == TM_COEF_POINT) {
#pragma unroll
            for (int b = 0; b < B; ++b)
#pragma unroll
              for (int h = 0; h < H; ++h) dpc[b][h] = dpc[b][h] + wdet * sn[h] * Nq[b];
          } else if (args.coef_kind == TM_COEF_ELEMENT) {
            dce = dce + wdet * sn[0];
          }
          cq = Num<R>::from_float(1.f);  // phi already carries f
        }
        if constexpr (!L::kLoad) {
          if (args.coef_kind == TM_COEF_ELEMENT) dce = dce + wdet * phi;
          else if (args.coef_kind == TM_COEF_QUAD && out_dc) out_dc[(int64_t)pair * Q + q] = tm_store<T, R>(wdet * phi);
          else if (args.coef_kind == TM_COEF_POINT) {
#pragma unroll
            for (int b = 0; b < B; ++b) dpc[b][0] = dpc[b][0] + wdet * phi * Nq[b];
          }
        }
        if (out_dX) {
          // A = w c |det J| (phi I - P^T M) J^-1 ; dX += dN A^T
          const R cw = wdet * cq;
          R C[D][D];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) {
              R s = Num<R>::zero();
#pragma unroll
              for (int b = 0; b < B; ++b) s = s + P[b][i] * M[b][j];
              C[i][j] = (i == j ? phi : Num<R>::zero()) - s;
            }
          R A[D][D];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) {
              R s = Num<R>::zero();
#pragma unroll
              for (int k = 0; k < D; ++k) s = s + C[i][k] * Jinv[k][j];
              A[i][j] = cw * s;
            }
#pragma unroll
          for (int b = 0; b < B; ++b)
#pragma unroll
            for (int j = 0; j < D; ++j) {
              R s = Num<R>::zero();
#pragma unroll
              for (int i = 0; i < D; ++i) s = s + dNq[b * D + i] * A[j][i];
              dX[b][j] = dX[b][j] + s;
            }
        }
      }
      if (out_dX) {
#pragma unroll
        for (int b = 0; b < B; ++b)
#pragma unroll
          for (int d = 0; d < D; ++d) out_dX[((int64_t)pair * B + b) * D + d] = tm_store<T, R>(dX[b][d]);
      }
      if (out_dc) {
        if (args.coef_kind == TM_COEF_ELEMENT) out_dc[pair] = tm_store<T, R>(dce);
        else if (args.coef_kind == TM_COEF_POINT) {
#pragma unroll
          for (int b = 0; b < B; ++b)
#pragma unroll
            for (int h = 0; h < PC; ++h) out_dc[((int64_t)pair * B + b) * PC + h] = tm_store<T, R>(dpc[b][h]);
        }
      }
    }
    __syncthreads();
  }
}

template <int EL, int FORM, int H, class R>
inline size_t patch_backward_smem_bytes(const tm_patch_plan& plan, int coef_kind, int chunk) {
  using L = Layout<EL, FORM, H>;
  constexpr int D = L::D, B = L::B;
  size_t n = kMaxQuad + kMaxQuad * B + kMaxQuad * B * D + (size_t)plan.max_vtx * D;
  if (coef_kind == TM_COEF_POINT) n += (size_t)plan.max_vtx * (L::kLoad ? H : 1);
  n += (size_t)chunk * L::SE;
  return n * sizeof(R) + (size_t)plan.max_rows * sizeof(int) + 16;
}

template <int EL, int FORM, int H, class T, class R>
int launch_patch_backward(const tm_patch_plan& plan, const tm_assemble_args& args, const tm_backward_args& bw,
                          cudaStream_t stream) {
  int dev = 0;
  cudaGetDevice(&dev);
  int max_optin = 0;
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int chunk = kThreads;
  size_t bytes = patch_backward_smem_bytes<EL, FORM, H, R>(plan, args.coef_kind, chunk);
  while (bytes > (size_t)max_optin && chunk > 1) {
    chunk /= 2;
    bytes = patch_backward_smem_bytes<EL, FORM, H, R>(plan, args.coef_kind, chunk);
  }
  if (bytes > (size_t)max_optin) return TM_ERR_INDEX;
  auto kern = patch_backward_kernel<EL, FORM, H, T, R>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return TM_ERR_CUDA;
  kern<<<plan.n_patches, kThreads, bytes, stream>>>(plan, args, bw, chunk);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

// Dispatch over form/H for one element type and one value type (computed in
// the same type).
template <int EL, class T>
int backward_element_as(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw,
                        cudaStream_t s) {
  constexpr int D = Elem<EL>::D;
  switch (a.form) {
    case TM_FORM_LAPLACE: return launch_patch_backward<EL, TM_FORM_LAPLACE, 1, T, T>(plan, a, bw, s);
    case TM_FORM_MASS: return launch_patch_backward<EL, TM_FORM_MASS, 1, T, T>(plan, a, bw, s);
    case TM_FORM_ELASTICITY: return launch_patch_backward<EL, TM_FORM_ELASTICITY, D, T, T>(plan, a, bw, s);
    case TM_FORM_LOAD:
      if (a.n_comp == 1) return launch_patch_backward<EL, TM_FORM_LOAD, 1, T, T>(plan, a, bw, s);
      if (a.n_comp == 2) return launch_patch_backward<EL, TM_FORM_LOAD, 2, T, T>(plan, a, bw, s);
      if (a.n_comp == 3) return launch_patch_backward<EL, TM_FORM_LOAD, 3, T, T>(plan, a, bw, s);
      return TM_ERR_UNSUPPORTED;
    default: return TM_ERR_UNSUPPORTED;
  }
}

template <int EL>
int backward_element(const tm_patch_plan& plan, const tm_assemble_args& a, const tm_backward_args& bw,
                     cudaStream_t s) {
  if (a.dtype == TM_F32) return backward_element_as<EL, float>(plan, a, bw, s);
  return backward_element_as<EL, double>(plan, a, bw, s);
}

}  // namespace tmg
