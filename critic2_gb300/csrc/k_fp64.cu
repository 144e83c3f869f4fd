// FP64 plain form of the GTO evaluator (critic2's calculate_mo_gto + the
// rho2 MO reduction, src/wfn_private@proc.F90:3161-3273 and 2546-2624) and
// the fused NCI epilogue (src/nci@proc.f90:565-571, 598-599 with the nucleus
// rule of src/fieldmod@proc.f90:1148-1154).
//
// Work decomposition: a block of 256 threads owns a tile of 32 points.
// Warp g computes the basis block chi(10) of primitive k0+g at all 32 points
// (so the primitive type is warp-uniform) into shared memory; then thread
// (g, p) contracts the 8-primitive chunk against the 8 MOs of group g for
// point p.  A pass covers 8 groups x MPG MOs; passes loop over the MOs.  The
// primitive cutoff is critic2's exactly: an atom is in the environment when
// d^2 <= spcutoff^2 and a primitive is skipped when sqrt(d^2) > dran; chunks
// where no point of the tile sees any primitive are skipped whole.
//
// GB300 executes FP64 at about 1.1 TFLOP/s, so this kernel is bound by the
// DFMA issue of the contraction (10 * nmo FMAs per in-range (point,
// primitive) pair); everything else is arranged around keeping the DFMA
// pipe fed: chi is built once per (point, primitive, pass) and shared by
// the 8 MO groups, coefficients are read as broadcast loads.
#include <cuda_runtime.h>

#include "c2g_internal.h"
#include "gto.cuh"
#include "points.cuh"

namespace c2g {
namespace {

constexpr int TP = kTilePoints;  // points per tile
constexpr int NG = 8;      // MO groups = warps
constexpr int KCH = 8;     // primitives per chunk (one per warp)
constexpr int NTHR = TP * NG;
constexpr int kPointKernelMax = 65536;  // index batches up to this size use k_eval_fp64_pt

// ------------------------------------------------------------------ sinks
struct RecSink {
  double *rec;
  int nr;
  __device__ void put(const DevWfn &, long idx, const double (&)[3], const double *r, int stride) const {
    for (int q = 0; q < nr; q++) rec[idx * nr + q] = r[q * stride];
  }
};

struct NciSink {
  double *crho, *cgrad;
  __device__ void put(const DevWfn &w, long idx, const double (&x)[3], const double *r, int stride) const {
    const double rho = r[0];
    double g0 = r[stride], g1 = r[2 * stride], g2 = r[3 * stride];
    // nucleus within 1e-5 bohr: gradient := 0
    bool nuc = false;
    for (int a = 0; a < w.natom && !nuc; a++) {
      const double4 A = w.atoms[a];
      const double dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
      nuc = (dx * dx + dy * dy + dz * dz) <= 1e-10;
    }
    if (nuc) g0 = g1 = g2 = 0.0;
    const double gmod = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
    double a6[6] = {r[4 * stride], r[5 * stride], r[6 * stride],
                    r[7 * stride], r[8 * stride], r[9 * stride]};
    double ev[3];
    eig3_sym_dev(a6, ev);
    const double cst = 6.18733545256027186;  // 2 (3 pi^2)^(1/3)
    cgrad[idx] = gmod / (cst * pow(fmax(rho, 1e-80), 4.0 / 3.0));
    crho[idx] = copysign(fabs(rho), ev[1]) * 100.0;
  }
  // Symmetric 3x3 eigenvalues (xx,yy,zz,xy,xz,yz), ascending; cyclic Jacobi.
  __device__ static void eig3_sym_dev(const double (&h)[6], double (&ev)[3]) {
    double a00 = h[0], a11 = h[1], a22 = h[2], a01 = h[3], a02 = h[4], a12 = h[5];
    for (int sweep = 0; sweep < 12; sweep++) {
      const double off = a01 * a01 + a02 * a02 + a12 * a12;
      const double dia = a00 * a00 + a11 * a11 + a22 * a22;
      if (off == 0.0 || off < 1e-34 * dia) break;
      // rotate (0,1)
      if (a01 != 0.0) {
        const double th = (a11 - a00) / (2.0 * a01);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        const double n00 = a00 - t * a01, n11 = a11 + t * a01;
        const double n02 = c * a02 - s * a12, n12 = s * a02 + c * a12;
        a00 = n00; a11 = n11; a01 = 0.0; a02 = n02; a12 = n12;
      }
      if (a02 != 0.0) {
        const double th = (a22 - a00) / (2.0 * a02);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        const double n00 = a00 - t * a02, n22 = a22 + t * a02;
        const double n01 = c * a01 - s * a12, n12 = s * a01 + c * a12;
        a00 = n00; a22 = n22; a02 = 0.0; a01 = n01; a12 = n12;
      }
      if (a12 != 0.0) {
        const double th = (a22 - a11) / (2.0 * a12);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        const double n11 = a11 - t * a12, n22 = a22 + t * a12;
        const double n01 = c * a01 - s * a02, n02 = s * a01 + c * a02;
        a11 = n11; a22 = n22; a12 = 0.0; a01 = n01; a02 = n02;
      }
    }
    double e0 = a00, e1 = a11, e2 = a22, t;
    if (e0 > e1) t = e0, e0 = e1, e1 = t;
    if (e1 > e2) t = e1, e1 = e2, e2 = t;
    if (e0 > e1) t = e0, e0 = e1, e1 = t;
    ev[0] = e0; ev[1] = e1; ev[2] = e2;
  }
};

// per-point partial record over the MPG MOs of one group (see kRec* layout)
template <int NC, int MPG, int NR, bool SPIN>
__device__ __forceinline__ void point_record(const double (&acc)[MPG][NC], const DevWfn &w, int mo0,
                                             double (&r)[NR]) {
#pragma unroll
  for (int q = 0; q < NR; q++) r[q] = 0.0;
#pragma unroll
  for (int m = 0; m < MPG; m++) {
    const double o = w.occ[mo0 + m];
    const double p0 = acc[m][0];
    r[0] += o * p0 * p0;
    if constexpr (NC > 1) {
      const double px = acc[m][1], py = acc[m][2], pz = acc[m][3];
      r[1] += 2.0 * o * p0 * px;
      r[2] += 2.0 * o * p0 * py;
      r[3] += 2.0 * o * p0 * pz;
      if constexpr (NC > 4) {
        r[4] += 2.0 * o * (p0 * acc[m][4] + px * px);
        r[5] += 2.0 * o * (p0 * acc[m][5] + py * py);
        r[6] += 2.0 * o * (p0 * acc[m][6] + pz * pz);
        r[7] += 2.0 * o * (p0 * acc[m][7] + px * py);
        r[8] += 2.0 * o * (p0 * acc[m][8] + px * pz);
        r[9] += 2.0 * o * (p0 * acc[m][9] + py * pz);
      }
      if constexpr (NR > kRecNci) {
        const double gk = px * px + py * py + pz * pz;
        r[10] += o * gk;
        if constexpr (NC > 4) {
          r[11] += o * (p0 * acc[m][4] - px * px);
          r[12] += o * (p0 * acc[m][7] - px * py);
          r[13] += o * (p0 * acc[m][8] - px * pz);
          r[14] += o * (p0 * acc[m][5] - py * py);
          r[15] += o * (p0 * acc[m][9] - py * pz);
          r[16] += o * (p0 * acc[m][6] - pz * pz);
        }
        if constexpr (SPIN) {
#pragma unroll
          for (int s = 0; s < 2; s++) {
            const double ws = (s == 0 ? w.wup : w.wdn)[mo0 + m];
            const int b = 17 + 11 * s;
            r[b] += ws * p0 * p0;
            r[b + 1] += 2.0 * ws * p0 * px;
            r[b + 2] += 2.0 * ws * p0 * py;
            r[b + 3] += 2.0 * ws * p0 * pz;
            r[b + 4] += ws * gk;
            if constexpr (NC > 4) {
              r[b + 5] += 2.0 * ws * (p0 * acc[m][4] + px * px);
              r[b + 6] += 2.0 * ws * (p0 * acc[m][5] + py * py);
              r[b + 7] += 2.0 * ws * (p0 * acc[m][6] + pz * pz);
              r[b + 8] += 2.0 * ws * (p0 * acc[m][7] + px * py);
              r[b + 9] += 2.0 * ws * (p0 * acc[m][8] + px * pz);
              r[b + 10] += 2.0 * ws * (p0 * acc[m][9] + py * pz);
            }
          }
        }
      }
    }
    if constexpr (NC == 1 && NR > kRecNci && SPIN) {
      // density only (nder = 0): the spin channels' rho
#pragma unroll
      for (int s = 0; s < 2; s++) r[17 + 11 * s] += (s == 0 ? w.wup : w.wdn)[mo0 + m] * p0 * p0;
    }
  }
}

template <int NDER, int MPG, int NR, bool SPIN, class Src, class Sink>
__global__ void __launch_bounds__(NTHR, 1) k_eval_fp64(DevWfn w, Src src, Sink sink, int ntiles) {
  constexpr int NC = NDER == 0 ? 1 : (NDER == 1 ? 4 : 10);
  constexpr int MOPASS = NG * MPG;
  __shared__ double s_x[3][TP];
  __shared__ int s_valid[TP];
  __shared__ long s_idx[TP];
  __shared__ __align__(16) double s_chi[KCH * 10 * TP];  // also the reduction buffer
  __shared__ double s_acc[NR * TP];
  __shared__ int s_any[KCH];
  static_assert(NG * 8 * TP <= KCH * 10 * TP, "reduction buffer");

  const int tid = threadIdx.x, p = tid & 31, g = tid >> 5;
  ntiles = src.tiles(ntiles);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    if (tid < TP) {
      double x[3] = {0.0, 0.0, 0.0};
      long idx = -1;
      const bool v = src.point(w, tile, tid, x, idx);
      s_x[0][tid] = x[0];
      s_x[1][tid] = x[1];
      s_x[2][tid] = x[2];
      s_valid[tid] = v;
      s_idx[tid] = idx;
    }
    for (int q = tid; q < NR * TP; q += NTHR) s_acc[q] = 0.0;
    if (!__syncthreads_or(tid < TP && s_valid[tid])) continue;
    const double px = s_x[0][p], py = s_x[1][p], pz = s_x[2][p];
    const bool pvalid = s_valid[p];

    for (int mo0 = 0; mo0 < w.nmo; mo0 += MOPASS) {
      double acc[MPG][NC];
#pragma unroll
      for (int m = 0; m < MPG; m++)
#pragma unroll
        for (int c = 0; c < NC; c++) acc[m][c] = 0.0;

      for (int k0 = 0; k0 < w.npri; k0 += KCH) {
        // basis block: warp g evaluates primitive k0+g at the 32 points
        const int ip = k0 + g;
        double chi[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) chi[c] = 0.0;
        bool in = false;
        if (ip < w.npri && pvalid) {
          const PrimF64 pr = w.prim[ip];
          const double4 A = w.atoms[pr.atom];
          const double dx = px - A.x, dy = py - A.y, dz = pz - A.z;
          const double dd = dx * dx + dy * dy + dz * dz;
          if (dd <= A.w) {
            const double dist = sqrt(dd);
            if (!(dist > pr.dran)) {
              in = true;
              const double ex = exp(-pr.e * (dist * dist));
              chi_eval<NC>(dx, dy, dz, pr.e, pr.lpack, ex, chi);
            }
          }
        }
#pragma unroll
        for (int c = 0; c < NC; c++) s_chi[(g * 10 + c) * TP + p] = chi[c];
        const unsigned any = __ballot_sync(0xffffffffu, in);
        if (p == 0) s_any[g] = (any != 0u);
        __syncthreads();
        // contraction: acc[m][c] += cmo(mo, prim) * chi(c)
#pragma unroll 1
        for (int kk = 0; kk < KCH; kk++) {
          if (!s_any[kk]) continue;
          const double2 *crow =
              reinterpret_cast<const double2 *>(w.cmo + (size_t)(k0 + kk) * w.nmo_pad + mo0 + g * MPG);
          double cm[MPG];
#pragma unroll
          for (int m = 0; m < MPG / 2; m++) {
            const double2 v = __ldg(crow + m);
            cm[2 * m] = v.x;
            cm[2 * m + 1] = v.y;
          }
#pragma unroll
          for (int c = 0; c < NC; c++) {
            const double xv = s_chi[(kk * 10 + c) * TP + p];
#pragma unroll
            for (int m = 0; m < MPG; m++) acc[m][c] = fma(cm[m], xv, acc[m][c]);
          }
        }
        __syncthreads();
      }
      // deterministic reduction of the 8 groups' partial records
      double r[NR];
      point_record<NC, MPG, NR, SPIN>(acc, w, mo0 + g * MPG, r);
#pragma unroll
      for (int q0 = 0; q0 < NR; q0 += NG) {
#pragma unroll
        for (int j = 0; j < NG; j++)
          if (q0 + j < NR) s_chi[(g * 8 + j) * TP + p] = r[q0 + j];
        __syncthreads();
        if (q0 + g < NR) {
          double sum = 0.0;
#pragma unroll
          for (int gg = 0; gg < NG; gg++) sum += s_chi[(gg * 8 + g) * TP + p];
          s_acc[(q0 + g) * TP + p] += sum;
        }
        __syncthreads();
      }
    }
    if (tid < TP && s_valid[tid]) {
      const double x[3] = {s_x[0][tid], s_x[1][tid], s_x[2][tid]};
      if (w.nedf) edf_add_record(w, x, s_acc + tid, TP, NR, SPIN);
      sink.put(w, s_idx[tid], x, s_acc + tid, TP);
    }
    __syncthreads();
  }
}

// Point-parallel FP64 form for small scattered batches (the Newton
// iterations): one block per point, one primitive per thread to build the
// basis block of up to 256 in-range primitives (compacted in primitive order
// by ballots, so the summation order is fixed), then one MO per thread (MPT
// MOs for nmo > 256) for the contraction, and a fixed-order block reduction
// of the 10 record sums.  GB300's FP64 rate per SM is low, so spreading a
// handful of points over many SMs is what makes these batches fast; the
// cutoffs are critic2's exactly, as in k_eval_fp64.
template <int MPT, class Src, class Sink>
__global__ void __launch_bounds__(256) k_eval_fp64_pt(DevWfn w, Src src, Sink sink) {
  constexpr int KC = 256;
  __shared__ double s_chi[KC * 10];
  __shared__ double s_d[KC * 4];
  __shared__ int s_k[KC];
  __shared__ int s_wn[8];
  __shared__ double s_red[8 * kRecNci];
  __shared__ double s_out[kRecNci];
  const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
  for (long t = blockIdx.x;; t += gridDim.x) {  // the list's points, grid-stride
    double x[3];
    long idx;
    if (!src.point(w, (int)(t / kTilePoints), (int)(t % kTilePoints), x, idx)) return;  // uniform per block
    double acc[MPT][10];
#pragma unroll
    for (int m = 0; m < MPT; m++)
#pragma unroll
      for (int c = 0; c < 10; c++) acc[m][c] = 0.0;
    for (int k0 = 0; k0 < w.npri; k0 += KC) {
      // the range tests of the chunk's primitives, those in range compacted
      // in primitive order, then their chi on the first threads (a warp
      // with one primitive in range would otherwise pay the whole FP64
      // exponential)
      const int ip = k0 + tid;
      double dx = 0.0, dy = 0.0, dz = 0.0, dd = 0.0;
      bool in = false;
      if (ip < w.npri) {
        const PrimF64 pr = w.prim[ip];
        const double4 A = w.atoms[pr.atom];
        dx = x[0] - A.x, dy = x[1] - A.y, dz = x[2] - A.z;
        dd = dx * dx + dy * dy + dz * dz;
        in = dd <= A.w && within_dran(dd, pr.dran);
      }
      const unsigned b = __ballot_sync(0xffffffffu, in);
      if (lane == 0) s_wn[wp] = __popc(b);
      __syncthreads();
      int base = 0, nact = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        base += i < wp ? s_wn[i] : 0;
        nact += s_wn[i];
      }
      if (in) {
        const int slot = base + __popc(b & ((1u << lane) - 1u));
        s_d[4 * slot] = dx, s_d[4 * slot + 1] = dy, s_d[4 * slot + 2] = dz, s_d[4 * slot + 3] = dd;
        s_k[slot] = ip;
      }
      __syncthreads();
      if (tid < nact) {
        const PrimF64 pr = w.prim[s_k[tid]];
        const double dist = sqrt(s_d[4 * tid + 3]);
        double chi[10];
        chi_eval<10>(s_d[4 * tid], s_d[4 * tid + 1], s_d[4 * tid + 2], pr.e, pr.lpack, exp(-pr.e * (dist * dist)),
                     chi);
#pragma unroll
        for (int c = 0; c < 10; c++) s_chi[tid * 10 + c] = chi[c];
      }
      __syncthreads();
      // threads without an MO skip the contraction (their sums stay zero)
#pragma unroll 2
      for (int j = 0; j < (tid < w.nmo ? nact : 0); j++) {
        const double *crow = w.cmo + (size_t)s_k[j] * w.nmo_pad;
        double ch[10];
#pragma unroll
        for (int c = 0; c < 10; c++) ch[c] = s_chi[j * 10 + c];
#pragma unroll
        for (int m = 0; m < MPT; m++) {
          const int mo = tid + 256 * m;
          const double cm = mo < w.nmo ? __ldg(crow + mo) : 0.0;
#pragma unroll
          for (int c = 0; c < 10; c++) acc[m][c] = fma(cm, ch[c], acc[m][c]);
        }
      }
      __syncthreads();
    }
    double r[kRecNci];
#pragma unroll
    for (int q = 0; q < kRecNci; q++) r[q] = 0.0;
#pragma unroll
    for (int m = 0; m < MPT; m++) {
      const int mo = tid + 256 * m;
      const double o = mo < w.nmo ? w.occ[mo] : 0.0;
      const double p0 = acc[m][0], px = acc[m][1], py = acc[m][2], pz = acc[m][3];
      r[0] += o * p0 * p0;
      r[1] += 2.0 * o * p0 * px;
      r[2] += 2.0 * o * p0 * py;
      r[3] += 2.0 * o * p0 * pz;
      r[4] += 2.0 * o * (p0 * acc[m][4] + px * px);
      r[5] += 2.0 * o * (p0 * acc[m][5] + py * py);
      r[6] += 2.0 * o * (p0 * acc[m][6] + pz * pz);
      r[7] += 2.0 * o * (p0 * acc[m][7] + px * py);
      r[8] += 2.0 * o * (p0 * acc[m][8] + px * pz);
      r[9] += 2.0 * o * (p0 * acc[m][9] + py * pz);
    }
#pragma unroll
    for (int q = 0; q < kRecNci; q++)
      for (int off = 16; off; off >>= 1) r[q] += __shfl_xor_sync(0xffffffffu, r[q], off);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < kRecNci; q++) s_red[wp * kRecNci + q] = r[q];
    __syncthreads();
    if (wp == 0) {
      double core_q = 0.0;  // EDF core, component `lane`
      if (w.nedf) {
        double core[10];
        edf_core_warp(w, x, core);
#pragma unroll
        for (int q = 0; q < 10; q++)
          if (q == lane) core_q = core[q];
      }
      if (tid < kRecNci) {
        double sum = 0.0;
        for (int i = 0; i < 8; i++) sum += s_red[i * kRecNci + tid];
        s_out[tid] = sum + core_q;
      }
    }
    __syncthreads();
    if (tid == 0) sink.put(w, idx, x, s_out, 1);
    __syncthreads();
  }
}

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    C2G_CUDA(cudaGetDevice(&dev));
    C2G_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// Per-point form: one block per point, a grid-stride loop over the list
// (at most 8 blocks per SM), so the launch does not grow with the list's
// capacity when its length lives on the device.
template <class Src, class Sink>
void launch_pt(const DevWfn &w, const Src &src, const Sink &sink, long maxn, cudaStream_t st) {
  const int grid = (int)std::min<long>(maxn, (long)num_sms() * 8);
  if (grid <= 0) return;
  if (w.nmo <= 256) k_eval_fp64_pt<1><<<grid, 256, 0, st>>>(w, src, sink);
  else if (w.nmo <= 512) k_eval_fp64_pt<2><<<grid, 256, 0, st>>>(w, src, sink);
  else k_eval_fp64_pt<4><<<grid, 256, 0, st>>>(w, src, sink);
  C2G_CUDA(cudaGetLastError());
}

template <class Src, class Sink>
void launch_any(const DevWfn &w, int nder, bool full, const Src &src, const Sink &sink, int ntiles,
                cudaStream_t st) {
  if (ntiles <= 0) return;
  const int grid = std::min(ntiles, num_sms() * 4);
  if (full) {
    if (w.spin) {
      if (nder == 2) k_eval_fp64<2, 4, kRecFull, true><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
      else if (nder == 1) k_eval_fp64<1, 4, kRecFull, true><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
      else k_eval_fp64<0, 4, kRecFull, true><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
    } else {
      if (nder == 2) k_eval_fp64<2, 4, kRecFull, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
      else if (nder == 1) k_eval_fp64<1, 4, kRecFull, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
      else k_eval_fp64<0, 4, kRecFull, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
    }
  } else {
    if (nder == 2) k_eval_fp64<2, 8, kRecNci, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
    else if (nder == 1) k_eval_fp64<1, 8, kRecNci, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
    else k_eval_fp64<0, 8, kRecNci, false><<<grid, NTHR, 0, st>>>(w, src, sink, ntiles);
  }
  C2G_CUDA(cudaGetLastError());
}

}  // namespace

void launch_fp64_points(const DevWfn &w, int n, const double *d_xyz, int nder, bool full,
                        double *d_rec, cudaStream_t st, bool wrap) {
  ListSrc src{d_xyz, n, wrap};
  RecSink sink{d_rec, full ? kRecFull : kRecNci};
  launch_any(w, nder, full, src, sink, (n + TP - 1) / TP, st);
}

void launch_fp64_index(const DevWfn &w, const double *d_x, const int *d_idx, const int *d_count,
                       int maxn, double *d_rec, cudaStream_t st) {
  IndexSrc src{d_x, d_idx, d_count};
  if (maxn <= 0) return;
  RecSink sink{d_rec, kRecNci};
  if (maxn <= kPointKernelMax && w.nmo <= 1024) {
    launch_pt(w, src, sink, maxn, st);
    return;
  }
  launch_any(w, 2, false, src, sink, (maxn + TP - 1) / TP, st);
}

void launch_fp64_nci_grid(const DevWfn &w, const GridSpec &g, double *d_crho, double *d_cgrad,
                          cudaStream_t st) {
  GridSrc src{g, (g.nstep[1] + 3) / 4, (g.nstep[2] + 7) / 8};
  NciSink sink{d_crho, d_cgrad};
  const long nt = (long)g.nstep[0] * src.ntj * src.ntk;
  launch_any(w, 2, false, src, sink, (int)nt, st);
}

void launch_fp64_nci_list(const DevWfn &w, const GridSpec &g, const int *d_list, const int *d_count,
                          int maxn, double *d_crho, double *d_cgrad, cudaStream_t st) {
  GridListSrc src{g, d_list, d_count};
  NciSink sink{d_crho, d_cgrad};
  if (w.nmo <= 1024) {
    // scattered re-check points: the per-point form spreads them over all SMs
    launch_pt(w, src, sink, maxn, st);
    return;
  }
  launch_any(w, 2, false, src, sink, (maxn + TP - 1) / TP, st);
}

}  // namespace c2g
