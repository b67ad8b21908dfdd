// Mesh-graph message-passing network (MPNN) kernels for the learned
// preconditioner: inference and training, BF16 operands on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation), hidden width 64.
//
// Graph: the rows of the condensed stiffness K_ii; edge weights are the
// symmetric normalised off-diagonal entries a_ij = K_ij / sqrt(K_ii K_jj)
// (a_ii = 0).  A hidden layer is
//     H_out = relu( H_in W_s + (A H_in) W_n + b )       (64 -> 64)
// computed per 64-row tile: the tile gathers A H_in for its rows (FP32
// accumulation, stored BF16), stages [H_in | A H_in] (64 x 128) and the
// stacked weights [W_s; W_n] (128 x 64) in shared memory, and each warp
// issues 8 k-steps x 8 n-tiles of mma.sync for 16 rows.  Backward kernels
// produce dH_in = dZ W_s^T + A (dZ W_n^T) and per-tile partial weight
// gradients [H_in | A H_in]^T dZ that a fixed-order reduction sums.
#include <cuda_bf16.h>

#include "tm_common.cuh"
#include "../../include/tensormesh_gb300.h"

namespace tmg {
namespace mp {

constexpr int F = 64;         // hidden channels
constexpr int TILE = 64;      // rows per CTA
constexpr int NT = 128;       // threads per CTA (4 warps, 16 rows each)
constexpr int LDA = 2 * F + 8;  // [H | AH] tile row stride (bf16 elements)
constexpr int LDW = 2 * F + 8;  // transposed weights Wt[n][k] row stride
constexpr int LDZ = F + 8;      // dZ tile row stride

typedef __nv_bfloat16 bf16;
typedef __nv_bfloat162 bf162;

TM_D uint32_t pack2(bf16 lo, bf16 hi) {
  uint32_t l = (uint32_t)__bfloat16_as_ushort(lo), h = (uint32_t)__bfloat16_as_ushort(hi);
  return l | (h << 16);
}
TM_D uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

TM_D void mma16816(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment (16x16) of a row-major bf16 tile: rows m0.., cols k0..
TM_D void frag_a(uint32_t* a, const bf16* s, int ld, int m0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  a[0] = ld32(s + (m0 + g) * ld + k0 + 2 * t);
  a[1] = ld32(s + (m0 + g + 8) * ld + k0 + 2 * t);
  a[2] = ld32(s + (m0 + g) * ld + k0 + 2 * t + 8);
  a[3] = ld32(s + (m0 + g + 8) * ld + k0 + 2 * t + 8);
}
// A fragment where A[m][k] = S[k][m] (S row-major): used for S^T dZ
TM_D void frag_a_trans(uint32_t* a, const bf16* s, int ld, int m0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  auto at = [&](int m, int k) { return s[(k0 + k) * ld + m0 + m]; };
  a[0] = pack2(at(g, 2 * t), at(g, 2 * t + 1));
  a[1] = pack2(at(g + 8, 2 * t), at(g + 8, 2 * t + 1));
  a[2] = pack2(at(g, 2 * t + 8), at(g, 2 * t + 9));
  a[3] = pack2(at(g + 8, 2 * t + 8), at(g + 8, 2 * t + 9));
}
// B fragment (16x8) where B[k][n] = T[n][k], T row-major (k contiguous)
TM_D void frag_b_nk(uint32_t* b, const bf16* s, int ld, int n0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  b[0] = ld32(s + (n0 + g) * ld + k0 + 2 * t);
  b[1] = ld32(s + (n0 + g) * ld + k0 + 2 * t + 8);
}
// B fragment where B[k][n] = S[k][n], S row-major (n contiguous)
TM_D void frag_b_kn(uint32_t* b, const bf16* s, int ld, int n0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  b[0] = pack2(s[(k0 + 2 * t) * ld + n0 + g], s[(k0 + 2 * t + 1) * ld + n0 + g]);
  b[1] = pack2(s[(k0 + 2 * t + 8) * ld + n0 + g], s[(k0 + 2 * t + 9) * ld + n0 + g]);
}

// Stage [H | A H] for rows row0..row0+63 (rows >= n are zero).  Warp w
// handles rows w, w+4, ...; lane l owns channels 2l, 2l+1.
TM_D void stage_h_ah(bf16* sA, int64_t n, int64_t row0, const int64_t* __restrict__ indptr,
                     const int32_t* __restrict__ idx, const float* __restrict__ aoff, const bf16* __restrict__ H) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int r = warp; r < TILE; r += NT / 32) {
    const int64_t row = row0 + r;
    float2 acc = make_float2(0.f, 0.f);
    bf162 h = __floats2bfloat162_rn(0.f, 0.f);
    if (row < n) {
      h = *reinterpret_cast<const bf162*>(H + row * F + 2 * lane);
      for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) {
        const float w = aoff[k];
        if (w == 0.f) continue;
        const float2 hj = __bfloat1622float2(*reinterpret_cast<const bf162*>(H + (int64_t)idx[k] * F + 2 * lane));
        acc.x += w * hj.x;
        acc.y += w * hj.y;
      }
    }
    *reinterpret_cast<bf162*>(sA + r * LDA + 2 * lane) = h;
    *reinterpret_cast<bf162*>(sA + r * LDA + F + 2 * lane) = __floats2bfloat162_rn(acc.x, acc.y);
  }
}

// H_out = act([H | AH] Wt^T + b); Wt is [64 out][128 in] bf16 (W transposed).
__global__ void __launch_bounds__(NT) layer_fwd(int64_t n, const int64_t* __restrict__ indptr,
                                                const int32_t* __restrict__ idx, const float* __restrict__ aoff,
                                                const bf16* __restrict__ Hin, const bf16* __restrict__ Wt,
                                                const float* __restrict__ bias, bf16* __restrict__ Hout, int relu) {
  __shared__ __align__(16) bf16 sA[TILE * LDA];
  __shared__ __align__(16) bf16 sW[F * LDW];
  const int64_t row0 = (int64_t)blockIdx.x * TILE;
  for (int i = threadIdx.x; i < F * 2 * F; i += NT) sW[(i / (2 * F)) * LDW + i % (2 * F)] = Wt[i];
  stage_h_ah(sA, n, row0, indptr, idx, aoff, Hin);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float c[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
#pragma unroll
  for (int ks = 0; ks < 8; ++ks) {
    uint32_t a[4];
    frag_a(a, sA, LDA, 16 * warp, 16 * ks, lane);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      uint32_t b[2];
      frag_b_nk(b, sW, LDW, 8 * nt, 16 * ks, lane);
      mma16816(c[nt], a, b);
    }
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int col = 8 * nt + 2 * t;
#pragma unroll
    for (int hf = 0; hf < 2; ++hf) {
      const int64_t row = row0 + 16 * warp + g + 8 * hf;
      if (row >= n) continue;
      float v0 = c[nt][2 * hf] + bias[col], v1 = c[nt][2 * hf + 1] + bias[col + 1];
      if (relu) {
        v0 = fmaxf(v0, 0.f);
        v1 = fmaxf(v1, 0.f);
      }
      *reinterpret_cast<bf162*>(Hout + row * F + col) = __floats2bfloat162_rn(v0, v1);
    }
  }
}

// Input lift: H0[i][c] = relu(x_i w0[c] + (A x)_i w1[c] + b[c]); also returns y = A x.
__global__ void input_fwd(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                          const float* __restrict__ aoff, const float* __restrict__ x, const float* __restrict__ w,
                          bf16* __restrict__ H0, float* __restrict__ y) {
  const int64_t row = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float s = 0.f;
  for (int64_t k = indptr[row] + lane; k < indptr[row + 1]; k += 32) s += aoff[k] * x[idx[k]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const float xi = x[row];
  if (lane == 0) y[row] = s;
  const int c = 2 * lane;
  float v0 = fmaxf(xi * w[c] + s * w[F + c] + w[2 * F + c], 0.f);
  float v1 = fmaxf(xi * w[c + 1] + s * w[F + c + 1] + w[2 * F + c + 1], 0.f);
  *reinterpret_cast<bf162*>(H0 + row * F + c) = __floats2bfloat162_rn(v0, v1);
}

// Readout, part 1: u_i = H_i . wr[0:64], t_i = H_i . wr[64:128]
__global__ void readout_dots(int64_t n, const bf16* __restrict__ H, const float* __restrict__ wr, float* __restrict__ u,
                             float* __restrict__ t) {
  const int64_t row = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float2 h = __bfloat1622float2(*reinterpret_cast<const bf162*>(H + row * F + 2 * lane));
  float a = h.x * wr[2 * lane] + h.y * wr[2 * lane + 1];
  float b = h.x * wr[F + 2 * lane] + h.y * wr[F + 2 * lane + 1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    u[row] = a;
    t[row] = b;
  }
}

// out_i = scale_i * (u_i + sum_j a_ij t_j)   (also used as y = A v with u = 0)
__global__ void gather_axpy(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                            const float* __restrict__ aoff, const float* __restrict__ u, const float* __restrict__ t,
                            const float* __restrict__ scale, float* __restrict__ out) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= n) return;
  float s = u ? u[row] : 0.f;
  for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) s += aoff[k] * t[idx[k]];
  out[row] = scale ? scale[row] * s : s;
}

// ---------------------------- backward ---------------------------------------
// Per tile: dZ = dHout * (Hout > 0)  [relu] ; partial dW (128 x 64) =
// [Hin | A Hin]^T dZ ; partial db = colsum(dZ) ; U = dZ Ws^T, T = dZ Wn^T
// (W is [128 in][64 out] bf16, row-major).
__global__ void __launch_bounds__(NT) layer_bwd_tile(int64_t n, const int64_t* __restrict__ indptr,
                                                     const int32_t* __restrict__ idx, const float* __restrict__ aoff,
                                                     const bf16* __restrict__ Hin, const bf16* __restrict__ Hout,
                                                     const float* __restrict__ dHout, const bf16* __restrict__ W,
                                                     float* __restrict__ part_dW, float* __restrict__ part_db,
                                                     float* __restrict__ U, float* __restrict__ T, int relu) {
  __shared__ __align__(16) bf16 sA[TILE * LDA];   // [Hin | A Hin]
  __shared__ __align__(16) bf16 sZ[TILE * LDZ];   // dZ
  __shared__ __align__(16) bf16 sW[2 * F * LDZ];  // W [128][64] row-major
  const int64_t row0 = (int64_t)blockIdx.x * TILE;
  for (int i = threadIdx.x; i < 2 * F * F; i += NT) sW[(i / F) * LDZ + i % F] = W[i];
  stage_h_ah(sA, n, row0, indptr, idx, aoff, Hin);
  for (int i = threadIdx.x; i < TILE * F; i += NT) {
    const int r = i / F, c = i % F;
    const int64_t row = row0 + r;
    float v = 0.f;
    if (row < n) {
      v = dHout[row * F + c];
      if (relu && !(__bfloat162float(Hout[row * F + c]) > 0.f)) v = 0.f;
    }
    sZ[r * LDZ + c] = __float2bfloat16_rn(v);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  // (1) partial dW: M = 128 (in channels), N = 64, K = 64 (rows); warp -> 32 M rows
  {
    float c[2][8][4];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
      for (int j = 0; j < 8; ++j) c[mi][j][0] = c[mi][j][1] = c[mi][j][2] = c[mi][j][3] = 0.f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      uint32_t a[2][4];
      frag_a_trans(a[0], sA, LDA, 32 * warp, 16 * ks, lane);
      frag_a_trans(a[1], sA, LDA, 32 * warp + 16, 16 * ks, lane);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b_kn(b, sZ, LDZ, 8 * nt, 16 * ks, lane);
        mma16816(c[0][nt], a[0], b);
        mma16816(c[1][nt], a[1], b);
      }
    }
    float* P = part_dW + (int64_t)blockIdx.x * (2 * F * F);
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
          const int m = 32 * warp + 16 * mi + g + 8 * hf, col = 8 * nt + 2 * t;
          P[m * F + col] = c[mi][nt][2 * hf];
          P[m * F + col + 1] = c[mi][nt][2 * hf + 1];
        }
  }
  if (threadIdx.x < F) {
    float s = 0.f;
    for (int r = 0; r < TILE; ++r) s += __bfloat162float(sZ[r * LDZ + threadIdx.x]);
    part_db[(int64_t)blockIdx.x * F + threadIdx.x] = s;
  }
  // (2) U = dZ Ws^T and T = dZ Wn^T : M = 64 rows (warp -> 16), N = 64, K = 64
  //     B[k][n] = W[n][k] for the half (Ws rows 0..63, Wn rows 64..127)
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float c[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      uint32_t a[4];
      frag_a(a, sZ, LDZ, 16 * warp, 16 * ks, lane);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        uint32_t b[2];
        frag_b_nk(b, sW + half * F * LDZ, LDZ, 8 * nt, 16 * ks, lane);
        mma16816(c[nt], a, b);
      }
    }
    float* O = half == 0 ? U : T;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        const int64_t row = row0 + 16 * warp + g + 8 * hf;
        if (row >= n) continue;
        const int col = 8 * nt + 2 * t;
        O[row * F + col] = c[nt][2 * hf];
        O[row * F + col + 1] = c[nt][2 * hf + 1];
      }
  }
}

// dHin[i] = U[i] + sum_j a_ij T[j]   (64 channels, warp per row)
__global__ void layer_bwd_gather(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                                 const float* __restrict__ aoff, const float* __restrict__ U, const float* __restrict__ T,
                                 float* __restrict__ dHin) {
  const int64_t row = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float2 acc = *reinterpret_cast<const float2*>(U + row * F + 2 * lane);
  for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) {
    const float w = aoff[k];
    if (w == 0.f) continue;
    const float2 v = *reinterpret_cast<const float2*>(T + (int64_t)idx[k] * F + 2 * lane);
    acc.x += w * v.x;
    acc.y += w * v.y;
  }
  *reinterpret_cast<float2*>(dHin + row * F + 2 * lane) = acc;
}

// Readout backward: g = dL/d(out pre-scale): dH[i] = g_i wr0 + (A g)_i wr1,
// partial dwr (per tile of 64 rows): [H^T g ; H^T (A g)].
__global__ void readout_bwd(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ idx,
                            const float* __restrict__ aoff, const bf16* __restrict__ H, const float* __restrict__ g,
                            const float* __restrict__ wr, float* __restrict__ dH, float* __restrict__ part) {
  __shared__ float s_part[2 * F];
  for (int i = threadIdx.x; i < 2 * F; i += blockDim.x) s_part[i] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float p0 = 0.f, p1 = 0.f, q0 = 0.f, q1 = 0.f;
  for (int r = warp; r < TILE; r += blockDim.x / 32) {
    const int64_t row = (int64_t)blockIdx.x * TILE + r;
    if (row >= n) continue;
    float ag = 0.f;
    for (int64_t k = indptr[row] + lane; k < indptr[row + 1]; k += 32) ag += aoff[k] * g[idx[k]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ag += __shfl_xor_sync(0xffffffffu, ag, o);
    const float gi = g[row];
    const int c = 2 * lane;
    dH[row * F + c] = gi * wr[c] + ag * wr[F + c];
    dH[row * F + c + 1] = gi * wr[c + 1] + ag * wr[F + c + 1];
    const float2 h = __bfloat1622float2(*reinterpret_cast<const bf162*>(H + row * F + c));
    p0 += h.x * gi;
    p1 += h.y * gi;
    q0 += h.x * ag;
    q1 += h.y * ag;
  }
  // fixed-order combine across warps: one warp at a time
  for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
    if (warp == w) {
      s_part[2 * lane] += p0;
      s_part[2 * lane + 1] += p1;
      s_part[F + 2 * lane] += q0;
      s_part[F + 2 * lane + 1] += q1;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 2 * F; i += blockDim.x) part[(int64_t)blockIdx.x * 2 * F + i] = s_part[i];
}

// Input layer backward: dZ0 = dH0 * (H0 > 0); partial [sum x dZ0 ; sum y dZ0 ; sum dZ0]
__global__ void input_bwd(int64_t n, const float* __restrict__ x, const float* __restrict__ y,
                          const bf16* __restrict__ H0, const float* __restrict__ dH0, float* __restrict__ part) {
  __shared__ float s_part[3 * F];
  for (int i = threadIdx.x; i < 3 * F; i += blockDim.x) s_part[i] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float a[6] = {0, 0, 0, 0, 0, 0};
  for (int r = warp; r < TILE; r += blockDim.x / 32) {
    const int64_t row = (int64_t)blockIdx.x * TILE + r;
    if (row >= n) continue;
    const int c = 2 * lane;
    const float2 h = __bfloat1622float2(*reinterpret_cast<const bf162*>(H0 + row * F + c));
    const float d0 = h.x > 0.f ? dH0[row * F + c] : 0.f;
    const float d1 = h.y > 0.f ? dH0[row * F + c + 1] : 0.f;
    a[0] += x[row] * d0;
    a[1] += x[row] * d1;
    a[2] += y[row] * d0;
    a[3] += y[row] * d1;
    a[4] += d0;
    a[5] += d1;
  }
  for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
    if (warp == w)
      for (int j = 0; j < 3; ++j) {
        s_part[j * F + 2 * lane] += a[2 * j];
        s_part[j * F + 2 * lane + 1] += a[2 * j + 1];
      }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 3 * F; i += blockDim.x) part[(int64_t)blockIdx.x * 3 * F + i] = s_part[i];
}

// out[j] = sum_t part[t][j], tiles in order
__global__ void reduce_tiles(int64_t n_tiles, int width, const float* __restrict__ part, float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= width) return;
  float s = 0.f;
  for (int64_t t = 0; t < n_tiles; ++t) s += part[t * width + j];
  out[j] = s;
}

}  // namespace mp
}  // namespace tmg

using tmg::mp::bf16;

static inline unsigned tiles_of(int64_t n) { return (unsigned)((n + tmg::mp::TILE - 1) / tmg::mp::TILE); }

extern "C" int tm_mpnn_input_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                 const float* x, const float* w, void* H0, float* y, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !aoff || !x || !w || !H0 || !y) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::mp::input_fwd<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, indptr, indices, aoff, x, w, (bf16*)H0, y);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_mpnn_layer_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                 const void* Hin, const void* Wt, const float* bias, void* Hout, int32_t relu,
                                 void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !aoff || !Hin || !Wt || !bias || !Hout) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::mp::layer_fwd<<<tiles_of(n), tmg::mp::NT, 0, s>>>(n, indptr, indices, aoff, (const bf16*)Hin, (const bf16*)Wt,
                                                          bias, (bf16*)Hout, relu);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_mpnn_readout_fwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                   const void* H, const float* wr, const float* scale, float* u, float* t,
                                   float* out, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  if (!indptr || !indices || !aoff || !H || !wr || !u || !t || !out) return TM_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::mp::readout_dots<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, (const bf16*)H, wr, u, t);
  tmg::mp::gather_axpy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, aoff, u, t, scale, out);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_mpnn_readout_bwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                   const void* H, const float* g, const float* wr, float* dH, float* part,
                                   float* dwr, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned nt = tiles_of(n);
  tmg::mp::readout_bwd<<<nt, 256, 0, s>>>(n, indptr, indices, aoff, (const bf16*)H, g, wr, dH, part);
  tmg::mp::reduce_tiles<<<1, 128, 0, s>>>(nt, 2 * tmg::mp::F, part, dwr);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_mpnn_layer_bwd(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                 const void* Hin, const void* Hout, const float* dHout, const void* W, int32_t relu,
                                 float* part_dW, float* part_db, float* U, float* T, float* dHin, float* dW,
                                 float* db, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned nt = tiles_of(n);
  tmg::mp::layer_bwd_tile<<<nt, tmg::mp::NT, 0, s>>>(n, indptr, indices, aoff, (const bf16*)Hin, (const bf16*)Hout,
                                                     dHout, (const bf16*)W, part_dW, part_db, U, T, relu);
  if (dHin)
    tmg::mp::layer_bwd_gather<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, indptr, indices, aoff, U, T, dHin);
  const int wdw = 2 * tmg::mp::F * tmg::mp::F;
  tmg::mp::reduce_tiles<<<(wdw + 255) / 256, 256, 0, s>>>(nt, wdw, part_dW, dW);
  tmg::mp::reduce_tiles<<<1, 64, 0, s>>>(nt, tmg::mp::F, part_db, db);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_mpnn_input_bwd(int64_t n, const float* x, const float* y, const void* H0, const float* dH0,
                                 float* part, float* dw, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned nt = tiles_of(n);
  tmg::mp::input_bwd<<<nt, 256, 0, s>>>(n, x, y, (const bf16*)H0, dH0, part);
  tmg::mp::reduce_tiles<<<1, 3 * tmg::mp::F, 0, s>>>(nt, 3 * tmg::mp::F, part, dw);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}

extern "C" int tm_gather_axpy_f32(int64_t n, const int64_t* indptr, const int32_t* indices, const float* aoff,
                                  const float* u, const float* t, const float* scale, float* out, void* stream) {
  if (n < 0) return TM_ERR_INVALID;
  if (n == 0) return TM_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tmg::mp::gather_axpy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, indptr, indices, aoff, u, t, scale, out);
  return cudaPeekAtLastError() == cudaSuccess ? TM_OK : TM_ERR_CUDA;
}
