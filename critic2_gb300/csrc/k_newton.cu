// Batched Newton critical-point refinement: critic2's field%newton
// (src/fieldmod@proc.f90:2238-2279) run for every live seed at once.
//
// Every iteration evaluates rho, grad and the Hessian at the live seeds
// (a compacted index list), then k_newton_step applies critic2's step
// logic per seed: converged when |grad| < gfnormeps (the gradient is zero
// within 1e-5 bohr of a nucleus, src/fieldmod@proc.f90:1148-1154), ier = 1
// on a singular Hessian, otherwise x -= H^-1 grad.  Seeds still live are
// appended to the next list.  Each seed's trajectory depends only on its
// own evaluations, so the list order (set by the atomic append) does not
// change any result.
//
// In the split-precision modes a seed first iterates on the tensor-core
// evaluator and moves to FP64 once its Newton step is shorter than
// kSwitchStep; convergence is only ever declared from an FP64 evaluation.
#include <cuda_runtime.h>

#include <vector>

#include "c2g_internal.h"
#include "k_tc.h"

namespace c2g {
namespace {

constexpr double kSwitchStep = 1e-5;  // bohr

struct NewtonCtx {
  const double4 *atoms;
  int natom;
  double cell_lo[3], cell_aa[3];
  double gfnormeps;
  int stall;        // > 0: stop after this many FP64 steps without a new minimum of |grad|
  double *gbest;    // per seed: smallest FP64 |grad| so far
  int *nstall;      // per seed: FP64 steps since that minimum
};

// mode: 0 = FP64 list, 1 = split list.  Split seeds whose step falls below
// kSwitchStep (or whose gradient already meets the threshold) move to the
// FP64 list; FP64 seeds follow critic2's newton exactly.
__global__ void k_newton_step(NewtonCtx c, const double *rec, double *x, const int *idx,
                              const int *count, int *ier, int *next64, int *count64, int *nextsp,
                              int *countsp, int mode) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *count) return;
  const int i = idx[t];
  const double *r = rec + (size_t)t * kRecNci;
  // the evaluated (wrapped) position, for the nucleus rule
  double xw[3];
  for (int j = 0; j < 3; j++) {
    double f = (x[3 * i + j] - c.cell_lo[j]) / c.cell_aa[j];
    xw[j] = x[3 * i + j];
    if (f < -1e-4 || f > 1.0 + 1e-4) {
      f -= floor(f);
      xw[j] = c.cell_lo[j] + f * c.cell_aa[j];
    }
  }
  bool nuc = false;
  for (int a = 0; a < c.natom && !nuc; a++) {
    const double4 A = c.atoms[a];
    const double dx = xw[0] - A.x, dy = xw[1] - A.y, dz = xw[2] - A.z;
    nuc = (dx * dx + dy * dy + dz * dz) <= 1e-10;
  }
  double g0 = r[1], g1 = r[2], g2 = r[3];
  if (nuc) g0 = g1 = g2 = 0.0;
  const double gmod = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
  if (mode == 0 && c.stall > 0 && !(gmod < c.gfnormeps)) {
    // |grad| stuck at the FP64 rounding floor above gfnormeps: the seed
    // would only end at maxit (ier = 2)
    if (gmod < c.gbest[i]) {
      c.gbest[i] = gmod;
      c.nstall[i] = 0;
    } else if (++c.nstall[i] >= c.stall) {
      ier[i] = 2;
      return;
    }
  }
  if (gmod < c.gfnormeps) {
    if (mode == 0) {
      ier[i] = 0;
    } else {
      next64[atomicAdd(count64, 1)] = i;  // confirm in FP64
    }
    return;
  }
  // symmetric inverse by cofactors; exactly singular -> ier = 1
  const double a = r[4], d = r[5], f = r[6], b = r[7], cc = r[8], e = r[9];
  const double A = d * f - e * e, B = cc * e - b * f, C = b * e - cc * d;
  const double det = a * A + b * B + cc * C;
  if (det == 0.0 || !isfinite(det)) {
    if (mode == 0) ier[i] = 1;
    else next64[atomicAdd(count64, 1)] = i;
    return;
  }
  const double D = a * f - cc * cc, E = b * cc - a * e, F = a * d - b * b;
  const double id = 1.0 / det;
  const double s0 = (A * g0 + B * g1 + C * g2) * id;
  const double s1 = (B * g0 + D * g1 + E * g2) * id;
  const double s2 = (C * g0 + E * g1 + F * g2) * id;
  x[3 * i] -= s0;
  x[3 * i + 1] -= s1;
  x[3 * i + 2] -= s2;
  const double step = sqrt(s0 * s0 + s1 * s1 + s2 * s2);
  if (mode == 0 || step < kSwitchStep) next64[atomicAdd(count64, 1)] = i;
  else nextsp[atomicAdd(countsp, 1)] = i;
}

__global__ void k_iota(int *v, int n, int *count, int *ier, double *gbest, int *nstall) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    v[i] = i;
    ier[i] = 2;
    gbest[i] = 1e300;
    nstall[i] = 0;
  }
  if (i == 0) *count = n;
}

}  // namespace

// Runs the batch; x (3n, device) in/out, ier (n, device) out.
void newton_batch_dev(Handle &h, int n, double *d_x, int *d_ier, double gfnormeps, int maxit,
                      int prec, cudaStream_t st) {
  if (n <= 0) return;
  const DevWfn &w = h.dev;
  NewtonCtx c{w.atoms, w.natom, {w.cell_lo[0], w.cell_lo[1], w.cell_lo[2]},
              {w.cell_aa[0], w.cell_aa[1], w.cell_aa[2]}, gfnormeps, h.newton_stall, nullptr, nullptr};
  int *buf = nullptr;
  double *rec = nullptr;
  C2G_CUDA(cudaMalloc(&buf, sizeof(int) * (5 * (size_t)n + 8)));
  cudaError_t er = cudaMalloc(&rec, sizeof(double) * (kRecNci + 1) * (size_t)n);
  if (er != cudaSuccess) {
    cudaFree(buf);
    fail(C2G_ERR_ALLOC, "cudaMalloc (newton records)");
  }
  int *l64[2] = {buf, buf + n}, *lsp[2] = {buf + 2 * n, buf + 3 * n};
  int *cnt = buf + 4 * n;  // cnt[0..1] fp64 counts, cnt[2..3] split counts
  c.nstall = buf + 4 * n + 8;
  c.gbest = rec + (size_t)kRecNci * n;
  try {
    const bool split = (prec != C2G_PREC_FP64);
    C2G_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * 8, st));
    k_iota<<<(n + 255) / 256, 256, 0, st>>>(split ? lsp[0] : l64[0], n, split ? cnt + 2 : cnt, d_ier, c.gbest,
                                            c.nstall);
    C2G_CUDA(cudaGetLastError());
    int cur = 0;
    int h64 = split ? 0 : n, hsp = split ? n : 0;
    for (int it = 0; it < maxit && (h64 + hsp) > 0; it++) {
      const int nxt = cur ^ 1;
      C2G_CUDA(cudaMemsetAsync(cnt + nxt, 0, sizeof(int), st));
      C2G_CUDA(cudaMemsetAsync(cnt + 2 + nxt, 0, sizeof(int), st));
      if (hsp > 0) {
        tc_points_index(h, prec, d_x, lsp[cur], cnt + 2 + cur, hsp, rec, st);
        k_newton_step<<<(hsp + 127) / 128, 128, 0, st>>>(c, rec, d_x, lsp[cur], cnt + 2 + cur, d_ier,
                                                         l64[nxt], cnt + nxt, lsp[nxt], cnt + 2 + nxt, 1);
        C2G_CUDA(cudaGetLastError());
      }
      if (h64 > 0) {
        launch_fp64_index(w, d_x, l64[cur], cnt + cur, h64, rec, st);
        k_newton_step<<<(h64 + 127) / 128, 128, 0, st>>>(c, rec, d_x, l64[cur], cnt + cur, d_ier,
                                                         l64[nxt], cnt + nxt, lsp[nxt], cnt + 2 + nxt, 0);
        C2G_CUDA(cudaGetLastError());
      }
      int hc[4];
      C2G_CUDA(cudaMemcpyAsync(hc, cnt, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
      C2G_CUDA(cudaStreamSynchronize(st));
      h64 = hc[nxt];
      hsp = hc[2 + nxt];
      cur = nxt;
    }
    if (split) tc_check_error(h);
  } catch (...) {
    cudaFree(buf);
    cudaFree(rec);
    throw;
  }
  cudaFree(buf);
  cudaFree(rec);
}

}  // namespace c2g
