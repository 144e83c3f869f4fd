// Kernels of the learned critical-point seed proposer.
//
// A small fully convolutional 3D network reads a coarse grid of the
// density (features derived from the NCI evaluator's sign(lambda2)*rho and
// s on that grid) and predicts, per voxel, four CP-type heat maps
// (non-nuclear maximum, bond, ring, cage) and a sub-voxel offset to the CP.
// Its seeds replace critic2's pair seeding (src/autocp@proc.f90:423-437) in
// front of the unchanged Newton + addcp stages; there is no counterpart of
// the network in the reference.
//
// Everything the network needs on the GPU is here: the convolution
// forward pass, its backward passes for the input and for the weights, the
// loss with its gradient, the dense targets, Adam, the input features and
// the seed extraction.  Tensors are channel-last FP32, x[b][d][h][w][c];
// convolutions are "same" (zero padding), stride 1, 3^3 or 1^3 taps, with
// weights stored w[tap][cin][cout] (tap = (kz*K + ky)*K + kx, kz along d).
// The network is small (~70k weights) and its convolutions have 4-32
// channels, so they run on the FP32 pipes: the weights of one output-channel
// tile sit in shared memory and are read as broadcast float4 loads, each
// thread keeps two voxels x 16 channels of accumulators.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "c2g_internal.h"
#include "../../include/critic2_gb300_cpseed.h"

namespace c2g {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

// ---------------------------------------------------------------- forward
// FLIP = false: y = conv(x, w) (+ bias), cin = CIN.
// FLIP = true : the input-gradient pass dx = conv(dy, flip(w)^T): the input
// is dy with CIN = the layer's cout channels and the output has the layer's
// cin channels; tap k reads w[KS^3-1-k] with cin and cout swapped.
// Optional epilogues: ReLU, and multiplication by (mask > 0) (the ReLU
// derivative of the layer that produced the pass's output channels).
template <int CIN, int COT, int KS, bool FLIP>
__global__ void __launch_bounds__(kThreads) k_conv(const float *__restrict__ x, int B, int D, int H, int W,
                                                   const float *__restrict__ wt, int cin_w, int cout_w,
                                                   const float *__restrict__ bias, int relu,
                                                   const float *__restrict__ mask, float *__restrict__ y,
                                                   int cout_total) {
  constexpr int NT = KS * KS * KS;
  constexpr int P = KS / 2;
  extern __shared__ float4 ws4[];
  float *ws = reinterpret_cast<float *>(ws4);  // [NT][CIN][COT]
  const int co0 = blockIdx.y * COT;
  for (int i = threadIdx.x; i < NT * CIN * COT; i += kThreads) {
    const int c = i % COT, ci = (i / COT) % CIN, k = i / (COT * CIN);
    float v;
    if (!FLIP) v = wt[((size_t)k * cin_w + ci) * cout_w + co0 + c];
    else v = wt[((size_t)(NT - 1 - k) * cin_w + (co0 + c)) * cout_w + ci];
    ws[i] = v;
  }
  __syncthreads();
  const long nvox = (long)B * D * H * W;
  const long v0 = 2L * ((long)blockIdx.x * kThreads + threadIdx.x);
  if (v0 >= nvox) return;
  const int w0 = (int)(v0 % W);
  long r = v0 / W;
  const int h = (int)(r % H);
  r /= H;
  const int d = (int)(r % D);
  const int b = (int)(r / D);
  float acc0[COT], acc1[COT];
#pragma unroll
  for (int c = 0; c < COT; c++) acc0[c] = acc1[c] = 0.f;
#pragma unroll 1
  for (int kz = 0; kz < KS; kz++) {
    const int zz = d + kz - P;
    if (zz < 0 || zz >= D) continue;
#pragma unroll 1
    for (int ky = 0; ky < KS; ky++) {
      const int yy = h + ky - P;
      if (yy < 0 || yy >= H) continue;
      const float *row = x + (((long)b * D + zz) * H + yy) * (long)W * CIN;
#pragma unroll
      for (int kx = 0; kx < KS; kx++) {
        const int xa = w0 + kx - P, xb = xa + 1;
        const bool ina = xa >= 0 && xa < W, inb = xb >= 0 && xb < W;
        const float *wk = ws + ((kz * KS + ky) * KS + kx) * CIN * COT;
#pragma unroll
        for (int c4 = 0; c4 < CIN / 4; c4++) {
          const float4 va = ina ? ld4(row + (long)xa * CIN + 4 * c4) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float4 vb = inb ? ld4(row + (long)xb * CIN + 4 * c4) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float a[4] = {va.x, va.y, va.z, va.w}, bb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const float4 *wr = reinterpret_cast<const float4 *>(wk + (4 * c4 + j) * COT);
#pragma unroll
            for (int q = 0; q < COT / 4; q++) {
              const float4 w4 = wr[q];
              acc0[4 * q + 0] = fmaf(a[j], w4.x, acc0[4 * q + 0]);
              acc0[4 * q + 1] = fmaf(a[j], w4.y, acc0[4 * q + 1]);
              acc0[4 * q + 2] = fmaf(a[j], w4.z, acc0[4 * q + 2]);
              acc0[4 * q + 3] = fmaf(a[j], w4.w, acc0[4 * q + 3]);
              acc1[4 * q + 0] = fmaf(bb[j], w4.x, acc1[4 * q + 0]);
              acc1[4 * q + 1] = fmaf(bb[j], w4.y, acc1[4 * q + 1]);
              acc1[4 * q + 2] = fmaf(bb[j], w4.z, acc1[4 * q + 2]);
              acc1[4 * q + 3] = fmaf(bb[j], w4.w, acc1[4 * q + 3]);
            }
          }
        }
      }
    }
  }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const long v = v0 + e;
    if (v >= nvox) break;
    float *out = y + v * cout_total + co0;
    const float *mk = mask ? mask + v * cout_total + co0 : nullptr;
#pragma unroll
    for (int q = 0; q < COT / 4; q++) {
      float o[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        float t = e == 0 ? acc0[4 * q + j] : acc1[4 * q + j];
        if (bias) t += bias[co0 + 4 * q + j];
        if (relu) t = fmaxf(t, 0.f);
        if (mk && !(mk[4 * q + j] > 0.f)) t = 0.f;
        o[j] = t;
      }
      *reinterpret_cast<float4 *>(out + 4 * q) = make_float4(o[0], o[1], o[2], o[3]);
    }
  }
}

// --------------------------------------------------------- weight gradient
// dw[k][ci][co] += sum_v x[v + tap offset][ci] * dy[v][co]; db[co] += sum_v
// dy[v][co].  Grid: (blocks, taps).  A block stages chunks of V voxels (x at
// the tap's offset, zero outside, and dy) in shared memory; thread tiles of
// 2 cin x 4 cout, the block's threads split into G groups over the chunk's
// voxels; partial sums are reduced across groups and added with atomics.
template <int CIN, int COUT, int KS>
__global__ void __launch_bounds__(kThreads) k_conv_wgrad(const float *__restrict__ x, const float *__restrict__ dy,
                                                         int B, int D, int H, int W, float *__restrict__ dw,
                                                         float *__restrict__ db) {
  constexpr int V = 64;
  constexpr int P = KS / 2;
  constexpr int NTILE = (CIN / 2) * (COUT / 4);
  static_assert(kThreads % NTILE == 0 && NTILE <= kThreads, "thread tiling");
  constexpr int G = kThreads / NTILE;
  __shared__ __align__(16) float xs[V * CIN];
  __shared__ __align__(16) float ds[V * COUT];
  __shared__ float red[kThreads * 8];
  const int k = blockIdx.y;
  const int kz = k / (KS * KS), ky = (k / KS) % KS, kx = k % KS;
  const int tile = threadIdx.x % NTILE, grp = threadIdx.x / NTILE;
  const int ci0 = 2 * (tile / (COUT / 4)), cq0 = 4 * (tile % (COUT / 4));
  const long nvox = (long)B * D * H * W;
  const long nchunk = (nvox + V - 1) / V;
  float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  float bacc[4] = {0.f, 0.f, 0.f, 0.f};
  const bool do_bias = db != nullptr && k == 0 && ci0 == 0;
  for (long ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
    __syncthreads();
    for (int i = threadIdx.x; i < V * CIN / 4; i += kThreads) {
      const int vv = i / (CIN / 4), c4 = i % (CIN / 4);
      const long v = ch * V + vv;
      float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
      if (v < nvox) {
        const int w0 = (int)(v % W);
        long r = v / W;
        const int h = (int)(r % H);
        r /= H;
        const int d = (int)(r % D), b = (int)(r / D);
        const int zz = d + kz - P, yy = h + ky - P, xx = w0 + kx - P;
        if (zz >= 0 && zz < D && yy >= 0 && yy < H && xx >= 0 && xx < W)
          val = ld4(x + ((((long)b * D + zz) * H + yy) * W + xx) * CIN + 4 * c4);
      }
      *reinterpret_cast<float4 *>(xs + vv * CIN + 4 * c4) = val;
    }
    for (int i = threadIdx.x; i < V * COUT / 4; i += kThreads) {
      const int vv = i / (COUT / 4), c4 = i % (COUT / 4);
      const long v = ch * V + vv;
      *reinterpret_cast<float4 *>(ds + vv * COUT + 4 * c4) =
          v < nvox ? ld4(dy + v * COUT + 4 * c4) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
#pragma unroll 4
    for (int vv = grp; vv < V; vv += G) {
      const float2 xv = *reinterpret_cast<const float2 *>(xs + vv * CIN + ci0);
      const float4 dv = *reinterpret_cast<const float4 *>(ds + vv * COUT + cq0);
      acc[0][0] = fmaf(xv.x, dv.x, acc[0][0]);
      acc[0][1] = fmaf(xv.x, dv.y, acc[0][1]);
      acc[0][2] = fmaf(xv.x, dv.z, acc[0][2]);
      acc[0][3] = fmaf(xv.x, dv.w, acc[0][3]);
      acc[1][0] = fmaf(xv.y, dv.x, acc[1][0]);
      acc[1][1] = fmaf(xv.y, dv.y, acc[1][1]);
      acc[1][2] = fmaf(xv.y, dv.z, acc[1][2]);
      acc[1][3] = fmaf(xv.y, dv.w, acc[1][3]);
      if (do_bias) {
        bacc[0] += dv.x;
        bacc[1] += dv.y;
        bacc[2] += dv.z;
        bacc[3] += dv.w;
      }
    }
  }
  // reduce over the G groups
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 8; j++) red[threadIdx.x * 8 + j] = acc[j / 4][j % 4];
  __syncthreads();
  if (grp == 0) {
    float s[8];
#pragma unroll
    for (int j = 0; j < 8; j++) s[j] = 0.f;
    for (int g = 0; g < G; g++)
#pragma unroll
      for (int j = 0; j < 8; j++) s[j] += red[(g * NTILE + tile) * 8 + j];
#pragma unroll
    for (int j = 0; j < 8; j++) atomicAdd(&dw[((long)k * CIN + ci0 + j / 4) * COUT + cq0 + j % 4], s[j]);
  }
  if (db != nullptr && k == 0) {
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; j++) red[threadIdx.x * 8 + j] = bacc[j];
    __syncthreads();
    if (grp == 0 && ci0 == 0) {
      float s[4] = {0.f, 0.f, 0.f, 0.f};
      for (int g = 0; g < G; g++)
#pragma unroll
        for (int j = 0; j < 4; j++) s[j] += red[(g * NTILE + tile) * 8 + j];
#pragma unroll
      for (int j = 0; j < 4; j++) atomicAdd(&db[cq0 + j], s[j]);
    }
  }
}

// ------------------------------------------------------------------- loss
// Per voxel, 8 output channels: 0-3 heat-map logits (non-nuclear maximum,
// bond, ring, cage) with weighted binary cross-entropy (positives weighted
// by pos_w), mean over voxels; 4-6 sub-voxel offsets with a squared error
// on the labelled voxels (target channel 7 = 1), weighted by off_w and
// averaged over them; channel 7 unused.  Writes the gradient, adds the loss.
__global__ void __launch_bounds__(kThreads) k_loss(const float *__restrict__ lg, const float *__restrict__ tg,
                                                   long nvox, float inv_nvox, float inv_npos, float pos_w,
                                                   float off_w, float *__restrict__ dlg, double *loss) {
  const long v = (long)blockIdx.x * kThreads + threadIdx.x;
  float l = 0.f;
  if (v < nvox) {
    const float4 a = ld4(lg + 8 * v), o = ld4(lg + 8 * v + 4);
    const float4 t = ld4(tg + 8 * v), to = ld4(tg + 8 * v + 4);
    const float z[4] = {a.x, a.y, a.z, a.w}, y[4] = {t.x, t.y, t.z, t.w};
    float g[8];
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float wgt = y[c] > 0.5f ? pos_w : 1.f;
      // log(1 + exp(-|z|)) + max(z, 0) - z y
      const float sp = log1pf(expf(-fabsf(z[c]))) + fmaxf(z[c], 0.f) - z[c] * y[c];
      l += wgt * sp * inv_nvox;
      const float sg = 1.f / (1.f + expf(-z[c]));
      g[c] = wgt * (sg - y[c]) * inv_nvox;
    }
    const bool lab = to.w > 0.5f;
    const float e[3] = {o.x - to.x, o.y - to.y, o.z - to.z};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      g[4 + c] = lab ? off_w * e[c] * inv_npos : 0.f;
      if (lab) l += 0.5f * off_w * e[c] * e[c] * inv_npos;
    }
    g[7] = 0.f;
    *reinterpret_cast<float4 *>(dlg + 8 * v) = make_float4(g[0], g[1], g[2], g[3]);
    *reinterpret_cast<float4 *>(dlg + 8 * v + 4) = make_float4(g[4], g[5], g[6], g[7]);
  }
  __shared__ float red[kThreads / 32];
  for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < kThreads / 32; i++) s += red[i];
    atomicAdd(loss, s);
  }
}

// Dense targets from a CP list cps[n][5] = (sample, fi, fj, fk, type): the
// 8 voxels around each CP get its type and their offset to it.  tgt must
// be zero on entry.
__global__ void k_targets(const float *__restrict__ cps, int n, int S, float *__restrict__ tgt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *c = cps + 5 * i;
  const int b = (int)c[0], typ = (int)c[4];
  const float f[3] = {c[1], c[2], c[3]};
  const int i0[3] = {(int)floorf(f[0]), (int)floorf(f[1]), (int)floorf(f[2])};
  if (typ < 0 || typ > 3) return;
  for (int corner = 0; corner < 8; corner++) {
    int ii[3];
    bool in = true;
    for (int a = 0; a < 3; a++) {
      ii[a] = i0[a] + ((corner >> a) & 1);
      in = in && ii[a] >= 0 && ii[a] < S;
    }
    if (!in) continue;
    float *t = tgt + 8 * ((((long)b * S + ii[0]) * S + ii[1]) * S + ii[2]);
    t[typ] = 1.f;
    t[4] = f[0] - ii[0];
    t[5] = f[1] - ii[1];
    t[6] = f[2] - ii[2];
    t[7] = 1.f;
  }
}

// Input features from an NCI grid (crho = sign(lambda2) rho * 100, cgrad =
// s): scaled log10 rho, sign(lambda2), scaled -log10 s, and a zero channel.
__global__ void k_features(const double *__restrict__ crho, const double *__restrict__ cgrad, long n,
                           float *__restrict__ x) {
  const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const double cr = crho[v];
  const double rho = fabs(cr) / 100.0;
  const float lr = (float)log10(fmax(rho, 1e-30));
  const float ls = (float)log10(fmax(cgrad[v], 1e-4));
  const float f0 = (fminf(fmaxf(lr, -12.f), 4.f) + 4.f) * 0.25f;
  const float f1 = cr > 0.0 ? 1.f : (cr < 0.0 ? -1.f : 0.f);
  const float f2 = -fminf(fmaxf(ls, -4.f), 2.f) * 0.5f;
  *reinterpret_cast<float4 *>(x + 4 * v) = make_float4(f0, f1, f2, 0.f);
}

// Seeds from the network's output on one S^3 grid.  mode 0: voxels whose
// largest heat-map logit exceeds thr; mode 1: ... and whose largest logit is
// not exceeded by that of any of its 26 neighbours (ties go to the lower
// index); mode 2: voxels where some CP type's logit exceeds thr and is a
// maximum of that type's map over the 26 neighbours; mode 3: as 2 over the 6
// face neighbours.  A seed sits at the voxel centre plus the predicted
// offset (clamped to 1.5 voxels); voxel (i,j,k) is at x0 + h (i, j, k).
__device__ __forceinline__ float max4(const float4 &a) { return fmaxf(fmaxf(a.x, a.y), fmaxf(a.z, a.w)); }

__global__ void k_seeds(const float *__restrict__ lg, int S, double x00, double x01, double x02, double h,
                        float thr, int mode, int cap, double *__restrict__ seeds, int *__restrict__ vox,
                        int *__restrict__ count) {
  const long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long n = (long)S * S * S;
  if (v >= n) return;
  const float4 a = ld4(lg + 8 * v);
  const float p = max4(a);
  if (!(p > thr)) return;
  const int i = (int)(v / ((long)S * S)), j = (int)((v / S) % S), k = (int)(v % S);
  if (mode >= 1) {
    // per-type candidates: channels above thr (mode >= 2), or the max (mode 1)
    bool cand[4] = {a.x > thr, a.y > thr, a.z > thr, a.w > thr};
    const float av[4] = {a.x, a.y, a.z, a.w};
    for (int di = -1; di <= 1; di++)
      for (int dj = -1; dj <= 1; dj++)
        for (int dk = -1; dk <= 1; dk++) {
          const int ii = i + di, jj = j + dj, kk = k + dk;
          if ((di | dj | dk) == 0 || ii < 0 || jj < 0 || kk < 0 || ii >= S || jj >= S || kk >= S) continue;
          if (mode == 3 && (di != 0) + (dj != 0) + (dk != 0) != 1) continue;
          const long u = ((long)ii * S + jj) * S + kk;
          const float4 b = ld4(lg + 8 * u);
          if (mode == 1) {
            const float q = max4(b);
            if (q > p || (q == p && u < v)) return;
          } else {
            const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int t = 0; t < 4; t++)
              if (bv[t] > av[t] || (bv[t] == av[t] && u < v)) cand[t] = false;
          }
        }
    if (mode >= 2 && !(cand[0] || cand[1] || cand[2] || cand[3])) return;
  }
  const float4 o = ld4(lg + 8 * v + 4);
  const float oi = fminf(fmaxf(o.x, -1.5f), 1.5f), oj = fminf(fmaxf(o.y, -1.5f), 1.5f),
              ok = fminf(fmaxf(o.z, -1.5f), 1.5f);
  const int slot = atomicAdd(count, 1);
  if (slot >= cap) return;
  seeds[3 * slot + 0] = x00 + h * (i + oi);
  seeds[3 * slot + 1] = x01 + h * (j + oj);
  seeds[3 * slot + 2] = x02 + h * (k + ok);
  vox[slot] = (int)v;
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ s, int n, float lr, float b1, float b2, float eps, float bc1,
                       float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float si = b2 * s[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  s[i] = si;
  p[i] -= lr * (mi / bc1) / (sqrtf(si / bc2) + eps);
}

// ------------------------------------------------------------- dispatch
template <int CIN, int COT, int KS, bool FLIP>
void conv_launch(const float *x, int B, int D, int H, int W, const float *w, int cin_w, int cout_w,
                 const float *bias, int relu, const float *mask, float *y, int cout_total, cudaStream_t st) {
  auto fn = k_conv<CIN, COT, KS, FLIP>;
  const int smem = KS * KS * KS * CIN * COT * 4;
  C2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const long nvox = (long)B * D * H * W;
  const long nthr = (nvox + 1) / 2;
  dim3 grid((unsigned)((nthr + kThreads - 1) / kThreads), (unsigned)(cout_total / COT));
  fn<<<grid, kThreads, smem, st>>>(x, B, D, H, W, w, cin_w, cout_w, bias, relu, mask, y, cout_total);
  C2G_CUDA(cudaGetLastError());
}

template <int KS, bool FLIP>
void conv_cin(int cin, const float *x, int B, int D, int H, int W, const float *w, int cin_w, int cout_w,
              const float *bias, int relu, const float *mask, float *y, int cout_total, cudaStream_t st) {
  const bool t16 = cout_total % 16 == 0;
  switch (cin) {
#define C2G_CONV_CASE(C)                                                                                  \
  case C:                                                                                                 \
    if (t16) conv_launch<C, 16, KS, FLIP>(x, B, D, H, W, w, cin_w, cout_w, bias, relu, mask, y, cout_total, st); \
    else conv_launch<C, 8, KS, FLIP>(x, B, D, H, W, w, cin_w, cout_w, bias, relu, mask, y, cout_total, st);      \
    break;
    C2G_CONV_CASE(4)
    C2G_CONV_CASE(8)
    C2G_CONV_CASE(16)
    C2G_CONV_CASE(32)
#undef C2G_CONV_CASE
    default:
      fail(C2G_ERR_UNSUPPORTED, "convolution input channels must be 4, 8, 16 or 32");
  }
}

void check_conv(int B, int D, int H, int W, int cin, int cout, int ksize) {
  if (B <= 0 || D <= 0 || H <= 0 || W <= 0) fail(C2G_ERR_ARG, "tensor dimensions must be positive");
  if (ksize != 1 && ksize != 3) fail(C2G_ERR_UNSUPPORTED, "kernel size must be 1 or 3");
  if (cin != 4 && cin != 8 && cin != 16 && cin != 32) fail(C2G_ERR_UNSUPPORTED, "cin must be 4, 8, 16 or 32");
  if (cout != 8 && cout != 16 && cout != 32) fail(C2G_ERR_UNSUPPORTED, "cout must be 8, 16 or 32");
}

template <int KS>
void wgrad_launch(int cin, int cout, const float *x, const float *dy, int B, int D, int H, int W, float *dw,
                  float *db, cudaStream_t st) {
  const long nvox = (long)B * D * H * W;
  const long nchunk = (nvox + 63) / 64;
  const int taps = KS * KS * KS;
  const long want = std::max(1L, (long)(4 * 152) / taps * 2);
  dim3 grid((unsigned)std::min(nchunk, want), (unsigned)taps);
#define C2G_WG(CI, CO)                                                                          \
  if (cin == CI && cout == CO) {                                                                \
    k_conv_wgrad<CI, CO, KS><<<grid, kThreads, 0, st>>>(x, dy, B, D, H, W, dw, db);              \
    C2G_CUDA(cudaGetLastError());                                                               \
    return;                                                                                     \
  }
  C2G_WG(4, 16) C2G_WG(4, 32) C2G_WG(8, 16) C2G_WG(8, 32) C2G_WG(16, 16) C2G_WG(16, 32) C2G_WG(32, 16)
  C2G_WG(32, 32) C2G_WG(32, 8) C2G_WG(16, 8) C2G_WG(8, 8) C2G_WG(4, 8)
#undef C2G_WG
  fail(C2G_ERR_UNSUPPORTED, "weight-gradient channel combination");
}

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_cs_conv3d(const float *x, int B, int D, int H, int W, int cin, const float *w, const float *bias,
                  int cout, int ksize, int relu, float *y, void *stream) {
  return guarded([&] {
    if (!x || !w || !y) fail(C2G_ERR_ARG, "null pointer");
    check_conv(B, D, H, W, cin, cout, ksize);
    if (W % 2) fail(C2G_ERR_UNSUPPORTED, "W must be even");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (ksize == 3) conv_cin<3, false>(cin, x, B, D, H, W, w, cin, cout, bias, relu, nullptr, y, cout, st);
    else conv_cin<1, false>(cin, x, B, D, H, W, w, cin, cout, bias, relu, nullptr, y, cout, st);
  });
}

int c2g_cs_conv3d_bwd_data(const float *dy, int B, int D, int H, int W, int cout, const float *w, int cin,
                           int ksize, const float *mask, float *dx, void *stream) {
  return guarded([&] {
    if (!dy || !w || !dx) fail(C2G_ERR_ARG, "null pointer");
    check_conv(B, D, H, W, cin, cout, ksize);
    if (cin % 8) fail(C2G_ERR_UNSUPPORTED, "input-gradient pass needs cin a multiple of 8");
    if (W % 2) fail(C2G_ERR_UNSUPPORTED, "W must be even");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (ksize == 3) conv_cin<3, true>(cout, dy, B, D, H, W, w, cin, cout, nullptr, 0, mask, dx, cin, st);
    else conv_cin<1, true>(cout, dy, B, D, H, W, w, cin, cout, nullptr, 0, mask, dx, cin, st);
  });
}

int c2g_cs_conv3d_bwd_weight(const float *x, const float *dy, int B, int D, int H, int W, int cin, int cout,
                             int ksize, float *dw, float *db, void *stream) {
  return guarded([&] {
    if (!x || !dy || !dw) fail(C2G_ERR_ARG, "null pointer");
    check_conv(B, D, H, W, cin, cout, ksize);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (ksize == 3) wgrad_launch<3>(cin, cout, x, dy, B, D, H, W, dw, db, st);
    else wgrad_launch<1>(cin, cout, x, dy, B, D, H, W, dw, db, st);
  });
}

int c2g_cs_loss(const float *logits, const float *tgt, long nvox, int npos, float pos_weight, float off_weight,
                float *dlogits, double *d_loss, void *stream) {
  return guarded([&] {
    if (!logits || !tgt || !dlogits || !d_loss) fail(C2G_ERR_ARG, "null pointer");
    if (nvox <= 0) fail(C2G_ERR_ARG, "nvox must be positive");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long nb = (nvox + kThreads - 1) / kThreads;
    k_loss<<<(unsigned)nb, kThreads, 0, st>>>(logits, tgt, nvox, 1.f / (float)nvox, 1.f / (float)std::max(1, npos),
                                               pos_weight, off_weight, dlogits, d_loss);
    C2G_CUDA(cudaGetLastError());
  });
}

int c2g_cs_targets(const float *d_cps, int ncp, int S, float *tgt, void *stream) {
  return guarded([&] {
    if (ncp < 0 || S <= 0 || !tgt || (ncp > 0 && !d_cps)) fail(C2G_ERR_ARG, "bad argument");
    if (ncp == 0) return;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_targets<<<(ncp + 127) / 128, 128, 0, st>>>(d_cps, ncp, S, tgt);
    C2G_CUDA(cudaGetLastError());
  });
}

int c2g_cs_features(const double *d_crho, const double *d_cgrad, long nvox, float *x, void *stream) {
  return guarded([&] {
    if (!d_crho || !d_cgrad || !x || nvox <= 0) fail(C2G_ERR_ARG, "bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_features<<<(unsigned)((nvox + 255) / 256), 256, 0, st>>>(d_crho, d_cgrad, nvox, x);
    C2G_CUDA(cudaGetLastError());
  });
}

int c2g_cs_seeds(const float *logits, int S, const double *x0, double h, float thresh_logit, int mode,
                 int cap, double *d_seeds, int *d_vox, int *d_count, void *stream) {
  return guarded([&] {
    if (!logits || !x0 || !d_seeds || !d_vox || !d_count || S <= 0 || cap < 0) fail(C2G_ERR_ARG, "bad argument");
    if (mode < 0 || mode > 3) fail(C2G_ERR_ARG, "seed mode must be 0-3");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const long n = (long)S * S * S;
    C2G_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
    k_seeds<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(logits, S, x0[0], x0[1], x0[2], h, thresh_logit,
                                                         mode, cap, d_seeds, d_vox, d_count);
    C2G_CUDA(cudaGetLastError());
  });
}

int c2g_cs_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                int t, void *stream) {
  return guarded([&] {
    if (!p || !g || !m || !v || n <= 0 || t <= 0) fail(C2G_ERR_ARG, "bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float bc1 = 1.f - std::pow(b1, (float)t), bc2 = 1.f - std::pow(b2, (float)t);
    k_adam<<<(n + 255) / 256, 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, bc1, bc2);
    C2G_CUDA(cudaGetLastError());
  });
}

}  // extern "C"
