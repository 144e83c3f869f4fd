// Split-precision GTO evaluator on the 5th-generation tensor cores.
//
// critic2's hot loop (src/wfn_private@proc.F90:3263-3268) is the product
//   phi_c(mo, p) = sum_k cmo(mo, k) * chi_c(k, p),  c = value, 3 first and
//   6 second derivatives,
// followed by the MO reduction of rho2 (src/wfn_private@proc.F90:2546-2624).
// Here it runs on tcgen05 MMAs with
//   M = 128 MOs (A = the coefficient tile, resident in tensor memory),
//   N = (component, point) pairs of a 32-point tile (B = the basis block chi
//       built in shared memory, one row per component and point),
//   K = one 32-byte row of primitives (16 bf16 or 8 tf32),
// in a 3-product split: A_hi*B_hi + A_hi*B_lo + A_lo*B_hi, FP32 accumulate.
// The tensor core's FP32 accumulation rounds toward zero, so every MMA into
// an accumulator shrinks it by up to an ulp of its size; the value
// component (the density) is protected from that bias: its hi*hi products
// rotate over four accumulators (K-step j into accumulator j mod 4) and its
// cross products have their own.  Per K-step eight or nine MMAs: hi*hi of
// components 0-7 (N = 256) or of component 0 alone (N = 32, accumulators
// 1-3) plus 1-7 (N = 224), hi*hi of 8-9 (N = 64), the two cross products
// of the value (N = 32) and those of components 1-9 (N = 128 + 160, into
// the main accumulator).  The accumulators (320 columns for the hi*hi
// products, 96 for three more value accumulators, 32 for the value's cross
// products) and 4 coefficient stages (16 columns each) fill the SM's 512
// TMEM columns.
//
// CTA roles (persistent, one CTA per SM, 12 warps):
//   warps 0-3  load the coefficient stage (L2 -> registers -> tcgen05.st into
//              TMEM) and run the epilogue: tcgen05.ld of phi, the
//              occupation-weighted products and the MO reduction (cross-lane
//              via shared memory) into per-quadrant partial sums;
//   warp 4     allocates TMEM; lane 0 issues the MMAs and commits;
//   warp 5     prepares each point tile: coordinates, per-atom offsets and
//              the list of K-stages that any point of the tile can see (a
//              stage is skipped only when every (point, primitive) pair in it
//              is beyond critic2's cutoff, so skipping changes no result),
//              ordered from the least to the most important one; after the
//              next tile's setup it runs the previous tile's sink: the sum
//              of the partial sums, FP64 accumulation over MO tiles, and the
//              NCI or record output;
//   warps 6-11 build the basis block chi (value, gradient, Hessian of every
//              primitive at the 32 points, split hi/lo) for one K-stage each.
// Hand-offs use mbarriers; tcgen05.commit releases shared stages and
// signals the accumulators.  Every wait is bounded (TcArgs::wait_ns, the
// handle's C2G_PARAM_WAIT_NS): on a timeout the CTA sets an error flag,
// stops, drains its MMAs and frees TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "gto.cuh"
#include "k_tc.h"
#include "points.cuh"
#include "ptx_sm100.h"

namespace c2g {

struct __align__(16) PrimTC {
  float al2e;      // alpha * log2(e)
  float alpha;     // alpha, rounded to FP32 ...
  float alpha_lo;  // ... and the remainder alpha - alpha_hi
  float dran;      // cutoff distance (0 for padding)
  int meta;        // atom << 12 | lx | ly << 4 | lz << 8
  int pad[3];
};

// Stage primitive data as the producer warp keeps it in shared memory: three
// 16-byte rows per primitive, read back as broadcast loads.
struct __align__(16) StageRow {
  float4 o;  // ox, oy, oz, g
  float4 l;  // lx, ly, lz, t
  float4 c;  // al2e, alpha, lp (bits), direct (bits)
};

struct TcKind {
  bool built = false;
  int kps = 0;        // primitives per K-stage
  int nstage = 0;
  int kpad = 0;
  PrimTC *prim = nullptr;
  uint8_t *c_hi = nullptr, *c_lo = nullptr;  // [mo_pad][kpad] elements
  // per-stage cutoff records: stage st owns entries [soff[st], soff[st+1])
  // = (atom as int bits, largest cutoff, smallest exponent) of each atom
  // with primitives in the stage
  int *soff = nullptr;
  float4 *sent = nullptr;
};

struct TcOperands {
  TcKind kind[2];  // 0 bf16, 1 tf32
  int mo_pad = 0, nmt = 0;
  float *occ = nullptr;
  int *err = nullptr;  // device error word
  std::vector<int> order;  // TC primitive order (indices into the handle's prims)
  std::vector<void *> allocs;
  double recheck_rel = -1.0;  // < 0: the mode's default (TF32x3 1e-4, BF16x3 1e-3)
  uint64_t wait_ns = 4000000000ull;  // limit of every pipeline wait of the split kernel
  int *scratch = nullptr;  // re-check list + counter, grown on demand
  uint8_t *atab = nullptr;  // per-CTA atom tables when they do not fit shared memory
  size_t atab_cap = 0;      // bytes
  size_t scratch_cap = 0;  // ints
};

namespace {
namespace K {
constexpr int NP = 32;     // points per tile
constexpr int MT = 128;    // MOs per tile (MMA M)
constexpr int NCOMP = 10;  // value, 3 first, 6 second derivatives
// The B operand has one row per (component, point) of the 32-point tile:
// row = component * 32 + point, 320 rows, so that an MMA covers several
// components at once (N = 32-256; small-N MMAs run at a fraction of the
// tensor pipe's rate).
constexpr int BROWS = NCOMP * NP;       // 320 B rows
constexpr int BPIECE = BROWS * 32;      // 10240 bytes: one (hi|lo) B operand
constexpr int STAGE = 2 * BPIECE;       // bytes of one K-stage (20480)
constexpr int NSTAGE = 6;  // shared-memory basis-block stages
constexpr int NCBUF = 4;   // coefficient buffers in TMEM
constexpr int NPROD = 6;
constexpr int W_MMA = 4, W_SETUP = 5, W_PROD0 = 6;
constexpr int NTHR = (W_PROD0 + NPROD) * 32;  // 384
constexpr uint32_t TMEM_COLS = 512;
// TMEM columns: the accumulators of the hi*hi products of the 10 components
// (320 columns, column = component * 32 + point), three more accumulators
// of the value's hi*hi products (96 columns), the accumulator of the value's
// cross products (hi*lo + lo*hi, 32 columns), then the coefficient buffers.
// Each value accumulator takes one truncating addition every fourth K-step,
// at a quarter of the size; the cross terms of the derivatives go into the
// main accumulator.
constexpr int NVACC = 4;                    // value accumulators
constexpr int DV0 = BROWS;                  // 320: value accumulators 1-3
constexpr int XCOL0 = DV0 + (NVACC - 1) * NP;  // 416: the value's cross products
constexpr int CBUF0 = XCOL0 + NP;           // 448
static_assert(CBUF0 + NCBUF * 16 <= (int)TMEM_COLS, "TMEM budget");
constexpr int RED = 81;  // padded row of the reduction buffer
constexpr int TAB = 4 * 13;  // axis-factor table: 4 primitives x (1 x + 4 y + 8 z values)
// barrier slots
// (B_CHI + stage buffer: the stage's basis block and its coefficients are in
// place, one arrival by the producer warp and one by each loader warp; the
// epilogue's partial sums are double-buffered: EPIFULL / EPIFREE per buffer)
constexpr int B_CHI = 0, B_EMPTY = 6, B_ACCFULL = 12, B_ACCEMPTY = 13, B_EPIFULL = 14, B_EPIFREE = 16,
              B_TREADY = 18, B_TFREE = 20, B_DRAIN = 22, NBAR = 23;
// One producer warp per stage buffer.  The buffer waits are mbarrier parity
// waits; with more producers than buffers the producer of stage g could wait
// for stage g - NSTAGE while stage g - 2 NSTAGE still holds the buffer, and
// the parity would alias.
static_assert(NSTAGE == NPROD, "one producer warp per stage buffer");
}  // namespace K

struct Mat3 {
  double m[9];
};

struct TcArgs {
  DevWfn w;
  const PrimTC *prim;
  const int *soff;
  const float4 *sent;
  const uint8_t *c_hi, *c_lo;
  const float *occ;
  int nstage, kpad, nmt, maskw;
  int *err;
  int *recheck, *recheck_count;
  int recheck_cap;
  float recheck_rel;
  unsigned long long *stage_count;  // total active (tile, stage) pairs, or null
  uint64_t wait_ns;                 // limit of every pipeline wait
  uint8_t *atab;                    // per-CTA atom tables in global memory, or null (shared memory)
  size_t atab_stride;               // bytes per CTA
};

struct Smem {
  uint64_t wait_ns;  // limit of every pipeline wait (TcArgs::wait_ns)
  uint8_t *stage;
  float *red, *part;
  double *acc;
  double *x;    // [2][32][3]
  long *idx;    // [2][32]
  float4 *dl;   // [2][32] offset from the tile reference point, w = valid
  uint64_t *bar;
  uint32_t *tmem;
  volatile int *abort;
  int *nact;    // [2]
  float *rad;   // [2] tile radius (max |delta|)
  uint8_t *key;    // [2][nstage] importance class of each stage (255 = inactive)
  uint16_t *list;  // [2][nstage] active stages, least important first
  float4 *off;   // [2][natom] o = reference - atom: (o_hi, |o|^2_hi)
  float4 *offl;  // [2][natom] (o - o_hi, |o|^2 - |o|^2_hi)
  float *dmin;   // [2][natom] lower bound of the tile-atom distance
  StageRow *rows;  // [NPROD][16] stage primitive data of each producer warp
  double4 *rowsd;  // [NPROD][16] centre and FP64 exponent of the same primitives (point-list tiles)
  float4 *tab;     // [NPROD][52] axis-factor tables of the brick path
  int *brick;      // [2] tile is a separable brick (see the setup warp)
};

// Bytes of the per-tile atom tables (off, offl, dmin for two tiles).
__host__ __device__ inline size_t atom_table_bytes(int natom) { return ((size_t)2 * natom * 36 + 15) / 16 * 16; }

// Shared-memory layout; the atom tables (offs[10-12]) are in it when
// atoms_smem, else in a per-CTA slice of global memory.
__host__ __device__ inline size_t smem_bytes(int natom, int maskw, bool atoms_smem, size_t *offs) {
  size_t o = 0;
  auto take = [&](size_t n, size_t al) {
    o = (o + al - 1) / al * al;
    size_t r = o;
    o += n;
    return r;
  };
  offs[0] = take((size_t)K::NSTAGE * K::STAGE, 1024);
  offs[1] = take(4 * 32 * K::RED * 4, 16);
  offs[2] = take(2 * 4 * 320 * 4, 16);
  offs[3] = take(10 * 32 * 8, 16);
  offs[4] = take(2 * 32 * 3 * 8, 16);
  offs[5] = take(2 * 32 * 8, 16);
  offs[6] = take(2 * 32 * 16, 16);
  offs[7] = take(K::NBAR * 8, 16);
  offs[8] = take(64, 16);
  offs[9] = take((size_t)2 * maskw * 32 * 3, 16);  // key (1 B) + list (2 B) per stage
  offs[13] = take((size_t)K::NPROD * 16 * (sizeof(StageRow) + sizeof(double4)), 16);
  offs[14] = take((size_t)K::NPROD * K::TAB * sizeof(float4), 16);
  const size_t at = atoms_smem ? take(atom_table_bytes(natom), 16) : 0;
  offs[10] = at;
  offs[11] = at + (size_t)2 * natom * 16;
  offs[12] = at + (size_t)4 * natom * 16;
  return o + 1024;  // slack for aligning the dynamic base
}

__device__ inline Smem carve(uint8_t *raw, const TcArgs &a) {
  const int natom = a.w.natom, maskw = a.maskw;
  uint8_t *base = (uint8_t *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
  size_t o[15];
  smem_bytes(natom, maskw, a.atab == nullptr, o);
  Smem s;
  s.stage = base + o[0];
  s.red = (float *)(base + o[1]);
  s.part = (float *)(base + o[2]);
  s.acc = (double *)(base + o[3]);
  s.x = (double *)(base + o[4]);
  s.idx = (long *)(base + o[5]);
  s.dl = (float4 *)(base + o[6]);
  s.bar = (uint64_t *)(base + o[7]);
  s.tmem = (uint32_t *)(base + o[8]);
  s.abort = (volatile int *)(base + o[8] + 4);
  s.nact = (int *)(base + o[8] + 8);
  s.rad = (float *)(base + o[8] + 16);
  s.key = (uint8_t *)(base + o[9]);
  s.list = (uint16_t *)(base + o[9] + (size_t)2 * maskw * 32);
  // the atom tables: in shared memory, or in this CTA's slice of a.atab
  uint8_t *ab = a.atab ? a.atab + (size_t)blockIdx.x * a.atab_stride - o[10] : base;
  s.off = (float4 *)(ab + o[10]);
  s.offl = (float4 *)(ab + o[11]);
  s.dmin = (float *)(ab + o[12]);
  s.rows = (StageRow *)(base + o[13]);
  s.rowsd = (double4 *)(base + o[13] + (size_t)K::NPROD * 16 * sizeof(StageRow));
  s.tab = (float4 *)(base + o[14]);
  s.brick = (int *)(base + o[8] + 24);
  s.wait_ns = a.wait_ns;
  return s;
}

// Bounded wait by one lane, result broadcast to the warp.
__device__ __forceinline__ bool warp_wait(const Smem &s, int bar, uint32_t parity, int *err) {
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    if (*s.abort) ok = 0;
    else if (!ptx::mbar_wait(&s.bar[bar], parity, s.wait_ns)) {
      ok = 0;
      *s.abort = 1;
      atomicOr(err, 1 << (bar < 31 ? bar : 31));
    }
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// A producer's wait for its stage buffer, taken just before the first
// store into the buffer, so that the part of the basis block computed in
// registers overlaps the MMAs that still read the buffer.
struct BufWait {
  uint64_t *bar;
  volatile int *abort;
  int *err;
  uint64_t wait_ns;
  uint32_t parity;
  int bit;
  bool need;
};

__device__ __forceinline__ bool buf_wait(const BufWait &w) {
  if (!w.need) return true;
  int ok = 1;
  if ((threadIdx.x & 31) == 0) {
    if (*w.abort) ok = 0;
    else if (!ptx::mbar_wait(w.bar, w.parity, w.wait_ns)) {
      ok = 0;
      *w.abort = 1;
      atomicOr(w.err, w.bit);
    }
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ bool thread_wait(const Smem &s, int bar, uint32_t parity, int *err) {
  if (*s.abort) return false;
  if (!ptx::mbar_wait(&s.bar[bar], parity, s.wait_ns)) {
    *s.abort = 1;
    atomicOr(err, 1 << (bar < 31 ? bar : 31));
    return false;
  }
  return true;
}

// 2^r for |r| <= 1/2 (+ a few ulp): 1 + r q(r) with q of degree 6, a
// weighted least-squares fit of (2^r - 1)/r on 400 Chebyshev nodes of
// [-0.501, 0.501] (relative error 2.7e-9 in exact arithmetic, FP32
// coefficients; gen_exp2.py); Horner in FP32 and a final fma keep the
// result within one ulp.
__device__ __forceinline__ float exp2_poly(float r) {
  float q = 1.51654758155928e-05f;
  q = fmaf(q, r, 1.546717103337869e-04f);
  q = fmaf(q, r, 1.3334084069356322e-03f);
  q = fmaf(q, r, 9.618036448955536e-03f);
  q = fmaf(q, r, 5.5504102259874344e-02f);
  q = fmaf(q, r, 2.4022650718688965e-01f);
  q = fmaf(q, r, 6.931471824645996e-01f);
  return fmaf(q, r, 1.f);
}

// 2^(xh + xl) for |xh| < 126, xl a correction below ulp(xh): n = rint(xh),
// 2^n by the exponent field, 2^((xh - n) + xl) by exp2_poly (xh - n is
// exact).  Within one ulp over the range; FP32's own exp2f is within two,
// and the rounding of a product argument alone (xl = 0) costs up to
// |x| * 2^-24 * ln 2 relative.
__device__ __forceinline__ float exp2_ff(float xh, float xl) {
  const float n = rintf(xh);
  const float p = exp2_poly((xh - n) + xl);
  const int ni = max(-126, min(127, (int)n));
  return __int_as_float(__float_as_int(p) + ni * 8388608);
}

// exp2(-(a * t)) with the rounding error of the product carried along
__device__ __forceinline__ float exp2_neg_prod(float a, float t) {
  const float xh = -a * t;
  return exp2_ff(xh, fmaf(-a, t, -xh));
}

// Factors of one Cartesian axis (see k_fp64.cu): with t = -2 alpha,
//   f0 = x^l, f1 = l x^(l-1) + t x^(l+1), f2 = l(l-1) x^(l-2) + t(2l+1) x^l + t^2 x^(l+2)
// Generic form (any l), used for stages that hold g or h functions.
__device__ __forceinline__ void axis_any(float x, int l, float t, float &f0, float &f1, float &f2) {
  float a = 1.f, b = 0.f, c = 0.f;
  for (int i = 0; i < l; i++) {
    c = b;
    b = a;
    a *= x;
  }
  const float p1 = a * x, p2 = p1 * x;
  f0 = a;
  f1 = fmaf(t, p1, (float)l * b);
  f2 = fmaf(t * t, p2, fmaf(t * (float)(2 * l + 1), a, (float)(l * (l - 1)) * c));
}

// Branch-free form for l <= 3 (s, p, d, f): x^l, x^(l-1), x^(l-2) are picked
// from the powers of x by the bits of l, so that the factors of several
// primitives can be evaluated as one straight-line block.
__device__ __forceinline__ void axis_f(float x, int l, float t, float &f0, float &f1, float &f2) {
  const float x2 = x * x;
  const float a = ((l & 1) ? x : 1.f) * ((l & 2) ? x2 : 1.f);  // x^l
  const int lm = l - 1;
  const float b = l ? ((lm & 1) ? x : 1.f) * ((lm & 2) ? x2 : 1.f) : 0.f;  // x^(l-1)
  const float c = (l >= 2) ? ((l == 3) ? x : 1.f) : 0.f;                   // x^(l-2)
  const float fl = (float)l;
  f0 = a;
  f1 = fmaf(t * x, a, fl * b);
  f2 = fmaf(a, fmaf(t * t, x2, t * (float)(2 * l + 1)), fl * (fl - 1.f) * c);
}

// Per (tile, primitive) part of the Gaussian.  With d = o + delta (o = tile
// reference - atom, delta = point - reference):
//   exp(-alpha |d|^2) = exp(-alpha |o|^2) * exp(-alpha (2 o.delta + |delta|^2)).
// The first factor G is computed once per tile from the float-float |o|^2
// and alpha with a compensated conversion to base 2 (u = arg*log2(e) carried
// as hi + lo, 2^-u = 2^-n * 2^-f with |f| <= 1/2); the per-point factor has
// a small argument, so its FP32 rounding stays small.  T = dran^2 - |o|^2
// turns critic2's cutoff d <= dran into 2 o.delta + |delta|^2 <= T.  When
// alpha (2|o|R + R^2) is large (tight primitives; R = tile radius) the
// per-point factor could overflow, and the primitive is evaluated directly
// from the float-float distance instead (G = 1, exponent alpha |d|^2).
struct StagePrim {
  float ox, oy, oz, lx, ly, lz;  // o = hi + lo
  float g, t, al2e, alpha;
  int lp, direct;
};

__device__ __forceinline__ StagePrim stage_prim(const PrimTC &pr, const float4 &o, const float4 &ol, float rad) {
  StagePrim q;
  q.ox = o.x, q.oy = o.y, q.oz = o.z, q.lx = ol.x, q.ly = ol.y, q.lz = ol.z;
  const float ooh = o.w, ool = ol.w;
  const float p = pr.alpha * ooh;
  float pe = fmaf(pr.alpha, ooh, -p);
  pe = fmaf(pr.alpha, ool, fmaf(pr.alpha_lo, ooh, pe));
  const float L1 = 1.44269502162933349609375f, L2 = 1.925963033500011079e-8f;
  const float u = p * L1;
  float ue = fmaf(p, L1, -u);
  ue = fmaf(p, L2, fmaf(pe, L1, ue));
  const float n = rintf(u);
  const float f = (u - n) + ue;
  const float on = sqrtf(ooh);
  q.direct = pr.alpha * (2.f * on * rad + rad * rad) > 60.f;
  q.g = q.direct ? 1.f : ((n > 250.f) ? 0.f : ldexpf(exp2_poly(-f), -(int)n));
  // cutoff threshold on t (factorised) or on |d|^2 (direct); -inf for padding
  q.t = pr.dran > 0.f ? (q.direct ? pr.dran * pr.dran : pr.dran * pr.dran - (ooh + ool)) : -INFINITY;
  q.al2e = pr.al2e;
  q.alpha = pr.alpha;
  q.lp = pr.meta & 0xfff;
  return q;
}

__device__ __forceinline__ StagePrim load_stage_prim(const StageRow *rows, int j) {
  const float4 o = rows[j].o, l = rows[j].l, c = rows[j].c;
  StagePrim q;
  q.ox = o.x, q.oy = o.y, q.oz = o.z, q.g = o.w;
  q.lx = l.x, q.ly = l.y, q.lz = l.z, q.t = l.w;
  q.al2e = c.x, q.alpha = c.y, q.lp = __float_as_int(c.z), q.direct = __float_as_int(c.w);
  return q;
}

__device__ __forceinline__ StagePrim bcast(const StagePrim &v, int j) {
  StagePrim q;
  q.ox = __shfl_sync(0xffffffffu, v.ox, j);
  q.oy = __shfl_sync(0xffffffffu, v.oy, j);
  q.oz = __shfl_sync(0xffffffffu, v.oz, j);
  q.lx = __shfl_sync(0xffffffffu, v.lx, j);
  q.ly = __shfl_sync(0xffffffffu, v.ly, j);
  q.lz = __shfl_sync(0xffffffffu, v.lz, j);
  q.g = __shfl_sync(0xffffffffu, v.g, j);
  q.t = __shfl_sync(0xffffffffu, v.t, j);
  q.al2e = __shfl_sync(0xffffffffu, v.al2e, j);
  q.alpha = __shfl_sync(0xffffffffu, v.alpha, j);
  q.lp = __shfl_sync(0xffffffffu, v.lp, j);
  q.direct = __shfl_sync(0xffffffffu, v.direct, j);
  return q;
}

// Point data: delta (offset from the tile reference), 2*delta, |delta|^2,
// and the point itself (FP64, for the point-list path).
struct PointD {
  float x, y, z, x2, y2, z2, dd;
  double px, py, pz;
  bool valid;
};

// chi (10 components) of one primitive at one point; zero beyond the cutoff
template <bool ANYL>
__device__ __forceinline__ void chi10(const StagePrim &q, const PointD &d, float (&chi)[10]) {
  const float dx = (q.ox + d.x) + q.lx, dy = (q.oy + d.y) + q.ly, dz = (q.oz + d.z) + q.lz;
  const float t = fmaf(q.ox, d.x2, fmaf(q.oy, d.y2, fmaf(q.oz, d.z2, d.dd)));
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float targ = q.direct ? d2 : t;
  const bool in = d.valid && (targ <= q.t);
  const float e = exp2_neg_prod(q.al2e, targ);
  const float ex = in ? q.g * e : 0.f;
  const float tt = -2.f * q.alpha;
  float x0, x1, x2, y0, y1, y2, z0, z1, z2;
  if constexpr (ANYL) {
    axis_any(dx, q.lp & 15, tt, x0, x1, x2);
    axis_any(dy, (q.lp >> 4) & 15, tt, y0, y1, y2);
    axis_any(dz, (q.lp >> 8) & 15, tt, z0, z1, z2);
  } else {
    axis_f(dx, q.lp & 15, tt, x0, x1, x2);
    axis_f(dy, (q.lp >> 4) & 15, tt, y0, y1, y2);
    axis_f(dz, (q.lp >> 8) & 15, tt, z0, z1, z2);
  }
  const float yz = y0 * z0 * ex, xz = x0 * z0 * ex, xy = x0 * y0 * ex;
  chi[0] = x0 * yz;
  chi[1] = x1 * yz;
  chi[2] = y1 * xz;
  chi[3] = z1 * xy;
  chi[4] = x2 * yz;
  chi[5] = y2 * xz;
  chi[6] = z2 * xy;
  const float x1e = x1 * ex;
  chi[7] = x1e * y1 * z0;
  chi[8] = x1e * z1 * y0;
  chi[9] = y1 * z1 * x0 * ex;
}

// chi (10 components) of one primitive at one point, with the Gaussian's
// argument alpha |x - A|^2 formed in FP64 from the point and the centre A =
// (ax, ay, az, alpha in FP64) and passed to exp2 as a float-float: the form
// of point lists (c2g_rho2, c2g_grd, meshes, Newton seeds), whose 32-point
// tiles can span several bohr, where the tile-factorised Gaussian of chi10
// would carry the FP32 rounding of a large per-point argument.  Zero beyond
// the cutoff (|x - A|^2 <= dran2).
template <bool ANYL>
__device__ __forceinline__ void chi10_exact(const StagePrim &q, const double4 &A, float dran2, const PointD &d,
                                            float (&chi)[10]) {
  const double ddx = d.px - A.x, ddy = d.py - A.y, ddz = d.pz - A.z;
  const double d2 = fma(ddx, ddx, fma(ddy, ddy, ddz * ddz));
  const bool in = d.valid && (d2 <= (double)dran2);
  const double xd = -(A.w * d2) * 1.4426950408889634;
  const float xh = (float)xd;
  const float ex = in ? exp2_ff(xh, (float)(xd - (double)xh)) : 0.f;
  const float dx = (float)ddx, dy = (float)ddy, dz = (float)ddz;
  const float tt = -2.f * q.alpha;
  float x0, x1, x2, y0, y1, y2, z0, z1, z2;
  if constexpr (ANYL) {
    axis_any(dx, q.lp & 15, tt, x0, x1, x2);
    axis_any(dy, (q.lp >> 4) & 15, tt, y0, y1, y2);
    axis_any(dz, (q.lp >> 8) & 15, tt, z0, z1, z2);
  } else {
    axis_f(dx, q.lp & 15, tt, x0, x1, x2);
    axis_f(dy, (q.lp >> 4) & 15, tt, y0, y1, y2);
    axis_f(dz, (q.lp >> 8) & 15, tt, z0, z1, z2);
  }
  const float yz = y0 * z0 * ex, xz = x0 * z0 * ex, xy = x0 * y0 * ex;
  chi[0] = x0 * yz;
  chi[1] = x1 * yz;
  chi[2] = y1 * xz;
  chi[3] = z1 * xy;
  chi[4] = x2 * yz;
  chi[5] = y2 * xz;
  chi[6] = z2 * xy;
  const float x1e = x1 * ex;
  chi[7] = x1e * y1 * z0;
  chi[8] = x1e * z1 * y0;
  chi[9] = y1 * z1 * x0 * ex;
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// chi = x0 + x1: TF32 pieces, each rounded to nearest.
__device__ __forceinline__ void split_tf32(float v, uint32_t &x0, uint32_t &x1) {
  x0 = tf32_rna(v);
  x1 = tf32_rna(v - __uint_as_float(x0));
}

// The same for a pair of values as BF16x2 words.
__device__ __forceinline__ void split_bf16(float a, float b, uint32_t &x0, uint32_t &x1) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  x0 = *reinterpret_cast<const uint32_t *>(&h);
  x1 = *reinterpret_cast<const uint32_t *>(&l);
}

// One 16-byte half of the 32-byte K-row of one point: PPB primitives,
// 10 components x (hi, lo) pieces staged in registers, then stored with
// 16-byte stores into the K-major no-swizzle canonical layout (8-row core
// matrices of 16 bytes; the two K-halves 128 bytes apart, 8-row groups 256
// bytes apart).
template <int KIND, bool ANYL>
__device__ __noinline__ bool produce_half(const StageRow *rows, const double4 *rowsd, int half, const PointD &d, uint8_t *dst,
                                          BufWait bw) {
  constexpr int PPB = KIND == 0 ? 8 : 4;  // primitives per 16-byte half row
  const int r = threadIdx.x & 31;
  uint32_t wv[10][2][4];
#pragma unroll
  for (int j = 0; j < PPB; j += (KIND == 0 ? 2 : 1)) {
    if constexpr (KIND == 0) {
      float c0[10], c1[10];
      chi10_exact<ANYL>(load_stage_prim(rows, half * PPB + j), rowsd[half * PPB + j], rows[half * PPB + j].l.w, d, c0);
      chi10_exact<ANYL>(load_stage_prim(rows, half * PPB + j + 1), rowsd[half * PPB + j + 1],
                        rows[half * PPB + j + 1].l.w, d, c1);
#pragma unroll
      for (int c = 0; c < 10; c++) split_bf16(c0[c], c1[c], wv[c][0][j >> 1], wv[c][1][j >> 1]);
    } else {
      float c0[10];
      chi10_exact<ANYL>(load_stage_prim(rows, half * PPB + j), rowsd[half * PPB + j], rows[half * PPB + j].l.w, d, c0);
#pragma unroll
      for (int c = 0; c < 10; c++) split_tf32(c0[c], wv[c][0][j], wv[c][1][j]);
    }
  }
  // B row of component c at point r = c * 32 + r, whose 8-row group is
  // 4c + (r >> 3)
  if (!buf_wait(bw)) return false;
  uint8_t *row = dst + (r >> 3) * 256 + half * 128 + (r & 7) * 16;
#pragma unroll
  for (int c = 0; c < 10; c++)
#pragma unroll
    for (int pc = 0; pc < 2; pc++)
      *reinterpret_cast<uint4 *>(row + pc * K::BPIECE + c * 1024) =
          make_uint4(wv[c][pc][0], wv[c][pc][1], wv[c][pc][2], wv[c][pc][3]);
  return true;
}

// Brick form of produce_half: per group of 4 primitives, the warp first
// tabulates the three Cartesian factors (f0, f1, f2 of the axis, and the
// axis's share of the exponent argument) for the tile's 1 x, 4 y and 8 z
// offsets, then every lane forms chi from the three entries of its point.
// The factors and the per-primitive data are the ones of chi10.
template <int KIND, bool ANYL>
__device__ __noinline__ bool produce_half_brick(const StageRow *rows, int half, const PointD &d, uint8_t *dst,
                                                float4 *tab, const float4 *dlt, BufWait bw) {
  constexpr int PPB = KIND == 0 ? 8 : 4;
  const int r = threadIdx.x & 31;
  const int jo = r >> 3, ko = r & 7;
  uint32_t wv[10][2][4];
#pragma unroll
  for (int g0 = 0; g0 < PPB; g0 += 4) {
    __syncwarp();
    for (int e = r; e < K::TAB; e += 32) {
      const int jp = e / 13, w = e - 13 * jp;
      const int j = half * PPB + g0 + jp;
      const float4 o = rows[j].o, l = rows[j].l, c = rows[j].c;
      const int lp = __float_as_int(c.z);
      const bool direct = __float_as_int(c.w) != 0;
      float oa, la, dd;
      int lax;
      if (w == 0) {
        oa = o.x, la = l.x, dd = dlt[0].x, lax = lp & 15;
      } else if (w < 5) {
        oa = o.y, la = l.y, dd = dlt[(w - 1) * 8].y, lax = (lp >> 4) & 15;
      } else {
        oa = o.z, la = l.z, dd = dlt[w - 5].z, lax = (lp >> 8) & 15;
      }
      const float da = (oa + dd) + la;
      const float arg = direct ? da * da : fmaf(oa, 2.f * dd, dd * dd);
      float f0, f1, f2;
      if constexpr (ANYL) axis_any(da, lax, -2.f * c.y, f0, f1, f2);
      else axis_f(da, lax, -2.f * c.y, f0, f1, f2);
      tab[e] = make_float4(f0, f1, f2, arg);
    }
    __syncwarp();
#pragma unroll
    for (int jp = 0; jp < 4; jp += (KIND == 0 ? 2 : 1)) {
      float cc[2][10];
#pragma unroll
      for (int q = 0; q < (KIND == 0 ? 2 : 1); q++) {
        const int j = half * PPB + g0 + jp + q;
        const float4 X = tab[(jp + q) * 13], Y = tab[(jp + q) * 13 + 1 + jo], Z = tab[(jp + q) * 13 + 5 + ko];
        const float4 o = rows[j].o, l = rows[j].l, c = rows[j].c;
        const float targ = (X.w + Y.w) + Z.w;
        const bool in = d.valid && (targ <= l.w);
        const float ex = in ? o.w * exp2_neg_prod(c.x, targ) : 0.f;
        const float yz = Y.x * Z.x * ex, xz = X.x * Z.x * ex, xy = X.x * Y.x * ex;
        cc[q][0] = X.x * yz;
        cc[q][1] = X.y * yz;
        cc[q][2] = Y.y * xz;
        cc[q][3] = Z.y * xy;
        cc[q][4] = X.z * yz;
        cc[q][5] = Y.z * xz;
        cc[q][6] = Z.z * xy;
        const float x1e = X.y * ex;
        cc[q][7] = x1e * Y.y * Z.x;
        cc[q][8] = x1e * Z.y * Y.x;
        cc[q][9] = Y.y * Z.y * X.x * ex;
      }
      const int wd = (g0 + jp) >> (KIND == 0 ? 1 : 0);
      if constexpr (KIND == 0) {
#pragma unroll
        for (int c = 0; c < 10; c++) split_bf16(cc[0][c], cc[1][c], wv[c][0][wd], wv[c][1][wd]);
      } else {
#pragma unroll
        for (int c = 0; c < 10; c++) split_tf32(cc[0][c], wv[c][0][wd], wv[c][1][wd]);
      }
    }
  }
  if (!buf_wait(bw)) return false;
  uint8_t *row = dst + (r >> 3) * 256 + half * 128 + (r & 7) * 16;
#pragma unroll
  for (int c = 0; c < 10; c++)
#pragma unroll
    for (int pc = 0; pc < 2; pc++)
      *reinterpret_cast<uint4 *>(row + pc * K::BPIECE + c * 1024) =
          make_uint4(wv[c][pc][0], wv[c][pc][1], wv[c][pc][2], wv[c][pc][3]);
  return true;
}

// Builds one K-stage of the basis block (lane = point row).  The stage's
// primitive data is loaded once (lane j holds primitive j) and broadcast.
template <int KIND>
__device__ __forceinline__ bool produce(const TcArgs &a, const Smem &s, int par, int stage_k, uint8_t *dst,
                                        const PointD &d, float rad, StageRow *rows, double4 *rowsd, float4 *tab,
                                        BufWait bw) {
  constexpr int KPS = KIND == 0 ? 16 : 8;
  const int r = threadIdx.x & 31;
  const bool brick = s.brick[par] != 0;
  int lmax = 0;
  if (r < KPS) {
    const PrimTC pr = a.prim[stage_k + r];
    const int at = pr.meta >> 12;
    const StagePrim q = stage_prim(pr, s.off[par * a.w.natom + at], s.offl[par * a.w.natom + at], rad);
    rows[r].o = make_float4(q.ox, q.oy, q.oz, q.g);
    // point-list tiles: the cutoff as dran^2 (chi10_exact); brick tiles: q.t
    rows[r].l = make_float4(q.lx, q.ly, q.lz, brick ? q.t : (pr.dran > 0.f ? pr.dran * pr.dran : -1.f));
    rows[r].c = make_float4(q.al2e, q.alpha, __int_as_float(q.lp), __int_as_float(q.direct));
    if (!brick) {
      const double4 A = a.w.atoms[at];
      rowsd[r] = make_double4(A.x, A.y, A.z, (double)pr.alpha + (double)pr.alpha_lo);
    }
    lmax = max(q.lp & 15, max((q.lp >> 4) & 15, (q.lp >> 8) & 15));
  }
  lmax = __reduce_max_sync(0xffffffffu, lmax);  // also orders the row writes before the reads
  // the buffer wait is taken inside the first half, before its stores
  bool ok = true;
  if (brick) {
    const float4 *dlt = s.dl + par * 32;
    for (int half = 0; half < 2 && ok; half++, bw.need = false) {
      if (lmax <= 3) ok = produce_half_brick<KIND, false>(rows, half, d, dst, tab, dlt, bw);
      else ok = produce_half_brick<KIND, true>(rows, half, d, dst, tab, dlt, bw);
    }
  } else {
    for (int half = 0; half < 2 && ok; half++, bw.need = false) {
      if (lmax <= 3) ok = produce_half<KIND, false>(rows, rowsd, half, d, dst, bw);
      else ok = produce_half<KIND, true>(rows, rowsd, half, d, dst, bw);
    }
  }
  __syncwarp();
  return ok;
}

// per-point outputs -----------------------------------------------------------
// v[q*stride] are the point's 10 sums (rho, grad, hess xx yy zz xy xz yz),
// FP32 when the molecule has one MO tile, FP64 accumulations otherwise.
struct TcRecSink {
  double *rec;
  template <class T>
  __device__ void put(const TcArgs &, long idx, const T *v, int stride) const {
#pragma unroll
    for (int q = 0; q < 10; q++) rec[idx * 10 + q] = (double)v[q * stride];
  }
};

__device__ void eig3_f64(double a00, double a11, double a22, double a01, double a02, double a12,
                         double (&ev)[3]) {
  for (int sweep = 0; sweep < 12; sweep++) {
    const double off = a01 * a01 + a02 * a02 + a12 * a12;
    const double dia = a00 * a00 + a11 * a11 + a22 * a22;
    if (off == 0.0 || off < 1e-34 * dia) break;
    if (a01 != 0.0) {
      const double th = (a11 - a00) / (2.0 * a01);
      const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
      const double n02 = c * a02 - s * a12, n12 = s * a02 + c * a12;
      a00 -= t * a01; a11 += t * a01; a01 = 0.0; a02 = n02; a12 = n12;
    }
    if (a02 != 0.0) {
      const double th = (a22 - a00) / (2.0 * a02);
      const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
      const double n01 = c * a01 - s * a12, n12 = s * a01 + c * a12;
      a00 -= t * a02; a22 += t * a02; a02 = 0.0; a01 = n01; a12 = n12;
    }
    if (a12 != 0.0) {
      const double th = (a22 - a11) / (2.0 * a12);
      const double t = (th >= 0.0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
      const double n01 = c * a01 - s * a02, n02 = s * a01 + c * a02;
      a11 -= t * a12; a22 += t * a12; a12 = 0.0; a01 = n01; a02 = n02;
    }
  }
  double e0 = a00, e1 = a11, e2 = a22, t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  if (e1 > e2) t = e1, e1 = e2, e2 = t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  ev[0] = e0; ev[1] = e1; ev[2] = e2;
}

// Same sweeps in FP32, for the points whose Hessian has a small eigenvalue.
__device__ void eig3_f32(float a00, float a11, float a22, float a01, float a02, float a12, float (&ev)[3]) {
  for (int sweep = 0; sweep < 8; sweep++) {
    const float off = a01 * a01 + a02 * a02 + a12 * a12;
    const float dia = a00 * a00 + a11 * a11 + a22 * a22;
    if (off == 0.f || off < 1e-14f * dia) break;
    if (a01 != 0.f) {
      const float th = (a11 - a00) / (2.f * a01);
      const float t = copysignf(1.f, th) / (fabsf(th) + sqrtf(th * th + 1.f));
      const float c = rsqrtf(t * t + 1.f), s = t * c;
      const float n02 = c * a02 - s * a12, n12 = s * a02 + c * a12;
      a00 -= t * a01; a11 += t * a01; a01 = 0.f; a02 = n02; a12 = n12;
    }
    if (a02 != 0.f) {
      const float th = (a22 - a00) / (2.f * a02);
      const float t = copysignf(1.f, th) / (fabsf(th) + sqrtf(th * th + 1.f));
      const float c = rsqrtf(t * t + 1.f), s = t * c;
      const float n01 = c * a01 - s * a12, n12 = s * a01 + c * a12;
      a00 -= t * a02; a22 += t * a02; a02 = 0.f; a01 = n01; a12 = n12;
    }
    if (a12 != 0.f) {
      const float th = (a22 - a11) / (2.f * a12);
      const float t = copysignf(1.f, th) / (fabsf(th) + sqrtf(th * th + 1.f));
      const float c = rsqrtf(t * t + 1.f), s = t * c;
      const float n01 = c * a01 - s * a02, n02 = s * a01 + c * a02;
      a11 -= t * a12; a22 += t * a12; a12 = 0.f; a01 = n01; a02 = n02;
    }
  }
  float e0 = a00, e1 = a11, e2 = a22, t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  if (e1 > e2) t = e1, e1 = e2, e2 = t;
  if (e0 > e1) t = e0, e0 = e1, e1 = t;
  ev[0] = e0; ev[1] = e1; ev[2] = e2;
}

// NCI point (src/nci@proc.f90:565-571, 598-599).  sign(lambda2) from the
// characteristic polynomial (Descartes' rule is exact for the real roots of
// a symmetric matrix) unless some eigenvalue is small relative to the
// Hessian's scale; those points get an FP32 eigen-solve, and where
// |lambda2| < 1e-3 max|lambda| the sign is decided by an FP64 eigen-solve;
// the ones with |lambda2| < recheck_rel * max|lambda| go to the FP64
// re-evaluation list.  rho^(4/3) is taken in FP64 where rho < 1e-4.
struct TcNciSink {
  double *crho, *cgrad;
  template <class T>
  __device__ void put(const TcArgs &a, long idx, const T *v, int stride) const {
    const float rf = (float)v[0];
    const float gx = (float)v[stride], gy = (float)v[2 * stride], gz = (float)v[3 * stride];
    const float gm = sqrtf(fmaf(gx, gx, fmaf(gy, gy, gz * gz)));
    const float cst = 6.18733545256027186f;  // 2 (3 pi^2)^(1/3)
    double s;
    if (rf >= 1e-4f) {
      s = (double)(gm / (cst * rf * cbrtf(rf)));
    } else {
      const double rr = fmax((double)v[0], 1e-80);
      s = (double)gm / (6.18733545256027186 * rr * cbrt(rr));
    }
    const float hxx = (float)v[4 * stride], hyy = (float)v[5 * stride], hzz = (float)v[6 * stride];
    const float hxy = (float)v[7 * stride], hxz = (float)v[8 * stride], hyz = (float)v[9 * stride];
    const float tr = hxx + hyy + hzz;
    const float c2 = hxx * hyy - hxy * hxy + hxx * hzz - hxz * hxz + hyy * hzz - hyz * hyz;
    const float det = hxx * (hyy * hzz - hyz * hyz) - hxy * (hxy * hzz - hyz * hxz) + hxz * (hxy * hyz - hyy * hxz);
    const float nrm = sqrtf(hxx * hxx + hyy * hyy + hzz * hzz + 2.f * (hxy * hxy + hxz * hxz + hyz * hyz));
    bool neg;
    if (fabsf(det) > 1e-3f * nrm * nrm * nrm) {
      // sign changes of (1, -tr, c2, -det), zeros skipped
      const float seq[4] = {1.f, -tr, c2, -det};
      int changes = 0;
      float prev = 1.f;
#pragma unroll
      for (int i = 1; i < 4; i++)
        if (seq[i] != 0.f) {
          if ((seq[i] > 0.f) != (prev > 0.f)) changes++;
          prev = seq[i];
        }
      neg = changes < 2;
    } else {
      float ef[3];
      eig3_f32(hxx, hyy, hzz, hxy, hxz, hyz, ef);
      neg = signbit(ef[1]);
      const float bigf = fmaxf(fabsf(ef[0]), fabsf(ef[2]));
      if (fabsf(ef[1]) < fmaxf(2e-3f, 2.f * a.recheck_rel) * bigf) {
        double ev[3];
        eig3_f64((double)v[4 * stride], (double)v[5 * stride], (double)v[6 * stride], (double)v[7 * stride],
                 (double)v[8 * stride], (double)v[9 * stride], ev);
        neg = signbit(ev[1]);
        const double big = fmax(fabs(ev[0]), fabs(ev[2]));
        if (fabs(ev[1]) < (double)a.recheck_rel * big && a.recheck) {
          const int slot = atomicAdd(a.recheck_count, 1);
          if (slot < a.recheck_cap) a.recheck[slot] = (int)idx;
        }
      }
    }
    const double rho = (double)v[0];
    crho[idx] = (neg ? -fabs(rho) : fabs(rho)) * 100.0;
    cgrad[idx] = s;
  }
};

// Hands a point's 10 valence sums to the sink, with the EDF core (FP64,
// gto.cuh) added first when the wavefunction has one.
template <class Sink, class T>
__device__ __forceinline__ void put_point(const TcArgs &a, const Sink &sink, long idx, const T *v, int stride,
                                          const double *xp) {
  if (a.w.nedf) {
    const double x[3] = {xp[0], xp[1], xp[2]};
    double r[10];
    edf_core(a.w, x, r);
#pragma unroll
    for (int k = 0; k < 10; k++) r[k] += (double)v[k * stride];
    sink.put(a, idx, r, 1);
  } else {
    sink.put(a, idx, v, stride);
  }
}

// s + e = a + b exactly (Knuth's two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// ------------------------------------------------------------------ kernel
template <int KIND, class Src, class Sink>
__global__ void __launch_bounds__(K::NTHR, 1) k_tc(TcArgs a, Src src, Sink sink, int ntiles) {
  extern __shared__ uint8_t smem_raw[];
  const Smem s = carve(smem_raw, a);
  constexpr int KPS = KIND == 0 ? 16 : 8;
  constexpr int ESZ = KIND == 0 ? 2 : 4;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int b = 0; b < K::NSTAGE; b++) {
      ptx::mbar_init(&s.bar[K::B_CHI + b], 1 + 4);  // the producer and the four loaders
      ptx::mbar_init(&s.bar[K::B_EMPTY + b], 1);
    }
    ptx::mbar_init(&s.bar[K::B_ACCFULL], 1);
    ptx::mbar_init(&s.bar[K::B_ACCEMPTY], 4);
    for (int p = 0; p < 2; p++) {
      ptx::mbar_init(&s.bar[K::B_EPIFULL + p], 4);
      ptx::mbar_init(&s.bar[K::B_EPIFREE + p], 1);
    }
    for (int p = 0; p < 2; p++) {
      ptx::mbar_init(&s.bar[K::B_TREADY + p], 1);
      ptx::mbar_init(&s.bar[K::B_TFREE + p], K::NPROD + 1 + 4);
    }
    ptx::mbar_init(&s.bar[K::B_DRAIN], 1);
    *s.abort = 0;
    ptx::mbar_fence_init();
  }
  for (int i = threadIdx.x; i < 320; i += K::NTHR) s.acc[i] = 0.0;
  if (warp == K::W_MMA) {
    ptx::tmem_alloc(s.tmem, K::TMEM_COLS);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *s.tmem;
  ntiles = src.tiles(ntiles);
  const int ntl = ntiles > (int)blockIdx.x ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;

  if (warp == K::W_SETUP) {
    // The sink of a tile (sum of the four quadrants' partial sums, FP64
    // accumulation over MO tiles, the NCI or record output) runs here, after
    // the next tile's setup, so that its FP64 work stays off the loader /
    // epilogue warps that feed the next tile's MMAs.  One lane per point.
    auto sink_tile = [&](int tt) -> bool {
      const int pp = tt & 1;
      const int p = lane;
      for (int mt = 0; mt < a.nmt; mt++) {
        const uint32_t uu = (uint32_t)tt * (uint32_t)a.nmt + (uint32_t)mt;
        // partial sums of pass uu in buffer uu & 1
        const int pb = (int)(uu & 1u);
        if (!warp_wait(s, K::B_EPIFULL + pb, (uu >> 1) & 1, a.err)) return false;
        const float *part = s.part + pb * 1280;
        // the four quadrants' partial sums of the point, summed in FP64
        double v4[10];
#pragma unroll
        for (int k = 0; k < 10; k++) {
          const int i = (p >> 3) * 80 + k * 8 + (p & 7);
          v4[k] = ((double)part[i] + (double)part[320 + i]) + ((double)part[640 + i] + (double)part[960 + i]);
        }
        const long idx = s.idx[pp * 32 + p];
        const double *xp = s.x + (pp * 32 + p) * 3;
        if (a.nmt == 1) {
          if (idx >= 0) put_point(a, sink, idx, v4, 1, xp);
        } else {
#pragma unroll
          for (int k = 0; k < 10; k++) s.acc[k * 32 + p] += v4[k];
          if (mt == a.nmt - 1) {
            if (idx >= 0) put_point(a, sink, idx, s.acc + p, 32, xp);
#pragma unroll
            for (int k = 0; k < 10; k++) s.acc[k * 32 + p] = 0.0;
          }
        }
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&s.bar[K::B_EPIFREE + pb]);
      }
      return true;
    };
    bool sink_ok = true;
    // ---------------------------------------------------------- tile setup
    for (int t = 0; t < ntl; t++) {
      const int par = t & 1;
      if (t >= 2 && !warp_wait(s, K::B_TFREE + par, ((t >> 1) - 1) & 1, a.err)) break;
      const int tile = (int)blockIdx.x + t * (int)gridDim.x;
      double x[3] = {0.0, 0.0, 0.0};
      long idx = -1;
      const bool v = src.point(a.w, tile, lane, x, idx);
      double *sx = s.x + (par * 32 + lane) * 3;
      sx[0] = x[0], sx[1] = x[1], sx[2] = x[2];
      s.idx[par * 32 + lane] = v ? idx : -1;
      const unsigned vm = __ballot_sync(0xffffffffu, v);
      const int nv = __popc(vm);
      double ref[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double sum = v ? x[c] : 0.0;
        for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        ref[c] = nv ? sum / nv : 0.0;
      }
      const float4 dl = v ? make_float4((float)(x[0] - ref[0]), (float)(x[1] - ref[1]), (float)(x[2] - ref[2]), 1.f)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
      s.dl[par * 32 + lane] = dl;
      // Separable brick: every valid point's offset is (x offset of lane 0,
      // y offset of lane 8*(lane/8), z offset of lane lane%8), as for the
      // 1 x 4 x 8 grid tiles of an axis-aligned grid.  Then each Cartesian
      // factor of a primitive takes 1, 4 and 8 distinct values in the tile.
      {
        const float bx = __shfl_sync(0xffffffffu, dl.x, 0);
        const float by = __shfl_sync(0xffffffffu, dl.y, lane & 24);
        const float bz = __shfl_sync(0xffffffffu, dl.z, lane & 7);
        const bool okb = !v || (dl.x == bx && dl.y == by && dl.z == bz);
        const bool br = __all_sync(0xffffffffu, okb);
        if (lane == 0) s.brick[par] = br ? 1 : 0;
      }
      float rad = v ? sqrtf(dl.x * dl.x + dl.y * dl.y + dl.z * dl.z) : 0.f;
      for (int o = 16; o; o >>= 1) rad = fmaxf(rad, __shfl_xor_sync(0xffffffffu, rad, o));
      float4 *off = s.off + par * a.w.natom;
      float4 *offl = s.offl + par * a.w.natom;
      float *dmn = s.dmin + par * a.w.natom;
      for (int at = lane; at < a.w.natom; at += 32) {
        const double4 A = a.w.atoms[at];
        const double ox = ref[0] - A.x, oy = ref[1] - A.y, oz = ref[2] - A.z;
        const double oo = ox * ox + oy * oy + oz * oz;
        const float hx = (float)ox, hy = (float)oy, hz = (float)oz, ho = (float)oo;
        off[at] = make_float4(hx, hy, hz, ho);
        offl[at] = make_float4((float)(ox - hx), (float)(oy - hy), (float)(oz - hz), (float)(oo - ho));
        dmn[at] = sqrtf(ho) - rad - 1e-3f;
      }
      if (lane == 0) s.rad[par] = rad;
      __syncwarp();
      // K-stages: a stage is active iff some primitive can reach some point.
      // Its importance class bounds the largest Gaussian factor it can give
      // in the tile, exp(-min alpha dmin^2); the active stages are listed
      // from the least to the most important one, so that the truncating
      // FP32 accumulators stay small for most of the accumulation.
      // One lane per stage, from the stage's per-atom records: the atom's
      // primitive with the smallest exponent has the largest cutoff, so the
      // stage is active iff that cutoff reaches the tile, and the bound is
      // that primitive's alpha dmin^2 (the same values as from every
      // primitive of the stage).
      uint8_t *key = s.key + par * a.maskw * 32;
      uint16_t *list = s.list + par * a.maskw * 32;
      for (int st0 = 0; st0 < a.maskw * 32; st0 += 32) {
        const int st = st0 + lane;
        uint8_t kv = 255;
        if (nv && st < a.nstage) {
          bool act = false;
          float arg = 3.0e38f;
          const int e1 = a.soff[st + 1];
          for (int e = a.soff[st]; e < e1; e++) {
            const float4 E = a.sent[e];
            const float dmr = dmn[__float_as_int(E.x)];
            if (dmr <= E.y) {
              act = true;
              const float dm = fmaxf(dmr, 0.f);
              arg = fminf(arg, E.z * dm * dm);
            }
          }
          if (act) kv = (uint8_t)fminf(15.f, arg * 0.5f);
        }
        key[st] = kv;
      }
      __syncwarp();
      int nact = 0;
      for (int cls = 15; cls >= 0; cls--) {
        for (int wd = 0; wd < a.maskw; wd++) {
          const int st = wd * 32 + lane;
          const bool hit = st < a.nstage && key[st] == cls;
          const unsigned bb = __ballot_sync(0xffffffffu, hit);
          if (hit) list[nact + __popc(bb & ((1u << lane) - 1u))] = (uint16_t)st;
          nact += __popc(bb);
        }
      }
      if (lane == 0) {
        s.nact[par] = nact;
        if (a.stage_count) atomicAdd(a.stage_count, (unsigned long long)nact);
      }
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&s.bar[K::B_TREADY + par]);
      if (t >= 1 && !(sink_ok = sink_tile(t - 1))) break;
    }
    if (sink_ok && ntl > 0) sink_tile(ntl - 1);
  } else if (warp == K::W_MMA) {
    // ------------------------------------------------------------ MMA issue
    if (lane == 0) {
      constexpr uint32_t fmt = KIND == 0 ? 1 : 2;
      constexpr uint32_t id_256 = ptx::make_idesc(fmt, K::MT, 256);  // components 0-7
      constexpr uint32_t id_224 = ptx::make_idesc(fmt, K::MT, 224);  // components 1-7
      constexpr uint32_t id_160 = ptx::make_idesc(fmt, K::MT, 160);  // components 5-9
      constexpr uint32_t id_128 = ptx::make_idesc(fmt, K::MT, 128);  // components 1-4
      constexpr uint32_t id_64 = ptx::make_idesc(fmt, K::MT, 64);    // components 8-9
      constexpr uint32_t id_32 = ptx::make_idesc(fmt, K::MT, 32);    // component 0
      auto mma = [](uint32_t d, uint32_t a_t, uint64_t b_d, uint32_t id, uint32_t acc) {
        if constexpr (KIND == 0) ptx::mma_bf16_ts(d, a_t, b_d, id, acc);
        else ptx::mma_tf32_ts(d, a_t, b_d, id, acc);
      };
      uint32_t g = 0, u = 0;
      bool ok = true;
      for (int t = 0; t < ntl && ok; t++) {
        const int par = t & 1;
        if (!(ok = thread_wait(s, K::B_TREADY + par, (t >> 1) & 1, a.err))) break;
        const int nact = s.nact[par];
        for (int mt = 0; mt < a.nmt && ok; mt++, u++) {
          if (u > 0) {
            if (!(ok = thread_wait(s, K::B_ACCEMPTY, (u - 1) & 1, a.err))) break;
            ptx::tc_fence_after();
          }
          for (int j = 0; j < nact; j++, g++) {
            const int b = g % K::NSTAGE, cb = g % K::NCBUF;
            if (!(ok = thread_wait(s, K::B_CHI + b, (g / K::NSTAGE) & 1, a.err))) break;
            ptx::tc_fence_after();
            const uint32_t a_hi = tmem + K::CBUF0 + cb * 16, a_lo = a_hi + 8;
            const uint32_t sb = ptx::smem_u32(s.stage + b * K::STAGE);
            const uint32_t acc0 = j > 0 ? 1u : 0u;
            {
              const uint32_t sh = sb, sl = sb + K::BPIECE;
              const uint32_t dcol = tmem, xcol = tmem + K::XCOL0;
              // B row r of the 320-row piece starts r / 8 row groups of 256
              // bytes in: rows 0, 32 (component 1), 160 (5), 256 (8)
              const uint64_t bh = ptx::smem_desc_kmajor(sh, 128, 256);
              const uint64_t bl = ptx::smem_desc_kmajor(sl, 128, 256);
              const uint64_t bh1 = ptx::smem_desc_kmajor(sh + 4 * 256, 128, 256);
              const uint64_t bl1 = ptx::smem_desc_kmajor(sl + 4 * 256, 128, 256);
              const uint64_t bh5 = ptx::smem_desc_kmajor(sh + 20 * 256, 128, 256);
              const uint64_t bl5 = ptx::smem_desc_kmajor(sl + 20 * 256, 128, 256);
              const uint64_t bh8 = ptx::smem_desc_kmajor(sh + 32 * 256, 128, 256);
              // hi*hi: the value of K-step j goes to value accumulator j mod 4
              // (0 = the main one, whose first write initialises components 0-7)
              const int va = j % K::NVACC;
              if (va == 0) {
                mma(dcol, a_hi, bh, id_256, acc0);
              } else {
                mma(tmem + K::DV0 + (va - 1) * K::NP, a_hi, bh, id_32, j >= K::NVACC ? 1u : 0u);
                mma(dcol + 32, a_hi, bh1, id_224, 1u);
              }
              mma(dcol + 256, a_hi, bh8, id_64, acc0);
              // cross products: the value's apart, components 1-9 into the
              // main accumulator (initialised above in the first K-step)
              mma(xcol, a_hi, bl, id_32, acc0);
              mma(xcol, a_lo, bh, id_32, 1u);
              mma(dcol + 32, a_hi, bl1, id_128, 1u);
              mma(dcol + 160, a_hi, bl5, id_160, 1u);
              mma(dcol + 32, a_lo, bh1, id_128, 1u);
              mma(dcol + 160, a_lo, bh5, id_160, 1u);
            }
            ptx::mma_commit(&s.bar[K::B_EMPTY + b]);
          }
          if (!ok) break;
          ptx::mma_commit(&s.bar[K::B_ACCFULL]);
        }
        if (ok) ptx::mbar_arrive(&s.bar[K::B_TFREE + par]);
      }
      // drain outstanding MMAs before the teardown
      ptx::mma_commit(&s.bar[K::B_DRAIN]);
      // (a bound of its own: tensor memory is freed only after the MMAs end)
      ptx::mbar_wait(&s.bar[K::B_DRAIN], 0, s.wait_ns > 2000000000ull ? s.wait_ns : 2000000000ull);
    }
  } else if (warp >= K::W_PROD0) {
    // -------------------------------------------------------- basis block
    const int pw = warp - K::W_PROD0;
    uint32_t g = 0;
    bool ok = true;
    for (int t = 0; t < ntl && ok; t++) {
      const int par = t & 1;
      if (!(ok = warp_wait(s, K::B_TREADY + par, (t >> 1) & 1, a.err))) break;
      const float4 d4 = s.dl[par * 32 + lane];
      PointD d;
      d.x = d4.x, d.y = d4.y, d.z = d4.z;
      d.x2 = 2.f * d4.x, d.y2 = 2.f * d4.y, d.z2 = 2.f * d4.z;
      d.dd = fmaf(d4.x, d4.x, fmaf(d4.y, d4.y, d4.z * d4.z));
      d.valid = d4.w > 0.f;
      {
        const double *xp = s.x + (par * 32 + lane) * 3;
        d.px = xp[0], d.py = xp[1], d.pz = xp[2];
      }
      const float rad = s.rad[par];
      const uint16_t *list = s.list + par * a.maskw * 32;
      const int nact = s.nact[par];
      for (int mt = 0; mt < a.nmt && ok; mt++) {
        for (int j = 0; j < nact && ok; j++, g++) {
          if ((int)(g % K::NPROD) != pw) continue;
          const int sk = list[j];
          const int b = g % K::NSTAGE;
          const int eb = K::B_EMPTY + b;
          const BufWait bw{&s.bar[eb], s.abort, a.err, s.wait_ns, ((g / K::NSTAGE) - 1) & 1u, 1 << (eb < 31 ? eb : 31),
                           g >= (uint32_t)K::NSTAGE};
          if (!(ok = produce<KIND>(a, s, par, sk * KPS, s.stage + b * K::STAGE, d, rad, s.rows + pw * 16,
                                   s.rowsd + pw * 16, s.tab + pw * K::TAB, bw)))
            break;
          ptx::fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) ptx::mbar_arrive(&s.bar[K::B_CHI + b]);
        }
      }
      __syncwarp();
      if (ok && lane == 0) ptx::mbar_arrive(&s.bar[K::B_TFREE + par]);
    }
  } else {
    // ----------------------------------------- coefficient loader + epilogue
    const int q = warp;  // TMEM lane quadrant
    const uint32_t lanebase = (uint32_t)(32 * q) << 16;
    uint32_t g = 0, u = 0;
    bool ok = true;
    float *red = s.red + q * 32 * K::RED;
    for (int t = 0; t < ntl && ok; t++) {
      const int par = t & 1;
      if (!(ok = warp_wait(s, K::B_TREADY + par, (t >> 1) & 1, a.err))) break;
      const int nact = s.nact[par];
      const uint16_t *list = s.list + par * a.maskw * 32;
      for (int mt = 0; mt < a.nmt && ok; mt++, u++) {
        const int mo = mt * K::MT + 32 * q + lane;
        const uint8_t *crow_hi = a.c_hi + (size_t)mo * a.kpad * ESZ;
        const uint8_t *crow_lo = a.c_lo + (size_t)mo * a.kpad * ESZ;
        for (int j = 0; j < nact && ok; j++, g++) {
          const int sk = list[j];
          const int cb = g % K::NCBUF;
          const uint4 h0 = __ldg(reinterpret_cast<const uint4 *>(crow_hi + (size_t)sk * 32));
          const uint4 h1 = __ldg(reinterpret_cast<const uint4 *>(crow_hi + (size_t)sk * 32 + 16));
          const uint4 l0 = __ldg(reinterpret_cast<const uint4 *>(crow_lo + (size_t)sk * 32));
          const uint4 l1 = __ldg(reinterpret_cast<const uint4 *>(crow_lo + (size_t)sk * 32 + 16));
          // buffer cb was last read by the MMAs of stage g - NCBUF
          if (g >= (uint32_t)K::NCBUF) {
            const uint32_t gp = g - K::NCBUF;
            if (!(ok = warp_wait(s, K::B_EMPTY + gp % K::NSTAGE, (gp / K::NSTAGE) & 1, a.err))) break;
          }
          const uint32_t hv[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
          const uint32_t lv[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
          ptx::tmem_st8(tmem + lanebase + K::CBUF0 + cb * 16, hv);
          ptx::tmem_st8(tmem + lanebase + K::CBUF0 + cb * 16 + 8, lv);
          ptx::tmem_wait_st();
          ptx::tc_fence_before();
          __syncwarp();
          // stage g's coefficients are in TMEM buffer cb
          if (lane == 0) ptx::mbar_arrive(&s.bar[K::B_CHI + g % K::NSTAGE]);
        }
        if (!ok) break;
        // ----- epilogue of this (point tile, MO tile)
        if (!(ok = warp_wait(s, K::B_ACCFULL, u & 1, a.err))) break;
        ptx::tc_fence_after();
        // partial-sum buffer u & 1 was read by the setup warp's sink of pass u - 2
        const int pb = (int)(u & 1u);
        if (u >= 2 && !(ok = warp_wait(s, K::B_EPIFREE + pb, ((u >> 1) - 1) & 1, a.err))) break;
        float *part = s.part + pb * 1280 + q * 320;
        if (nact > 0) {
          const float occ = a.occ[mo];
#pragma unroll 1
          for (int ch = 0; ch < 4; ch++) {
            uint32_t v[10][8], xv[8], dv[K::NVACC - 1][8];
            // points ch*8 .. ch*8+7
            const uint32_t dc = tmem + lanebase + ch * 8;
            const uint32_t xc = tmem + lanebase + K::XCOL0 + ch * 8;
#pragma unroll
            for (int c = 0; c < 10; c++) ptx::tmem_ld8(dc + c * K::NP, v[c]);
#pragma unroll
            ptx::tmem_ld8(xc, xv);
            // value accumulator c + 1 holds K-steps c + 1, c + 5, ...: written iff nact > c + 1
#pragma unroll
            for (int c = 0; c < K::NVACC - 1; c++) {
#pragma unroll
              for (int i = 0; i < 8; i++) dv[c][i] = 0u;
              if (nact > c + 1) ptx::tmem_ld8(tmem + lanebase + K::DV0 + c * K::NP + ch * 8, dv[c]);
            }
            ptx::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; j++) {
              // phi: the value accumulators summed exactly (two-sums), the
              // cross products (2^-11 of phi and below) added to the low part,
              // rounded once
              float sh = __uint_as_float(v[0][j]), sl = __uint_as_float(xv[j]);
#pragma unroll
              for (int c = 0; c < K::NVACC - 1; c++) {
                float e;
                two_sum(sh, __uint_as_float(dv[c][j]), sh, e);
                sl += e;
              }
              const float p0 = sh + sl;
              const float px = __uint_as_float(v[1][j]);
              const float py = __uint_as_float(v[2][j]);
              const float pz = __uint_as_float(v[3][j]);
              const float o2 = 2.f * occ, t0 = o2 * p0;
              const float ux = o2 * px, uy = o2 * py, uz = o2 * pz;
              float *rw = red + lane * K::RED + j;
              rw[0] = occ * p0 * p0;
              rw[8] = t0 * px;
              rw[16] = t0 * py;
              rw[24] = t0 * pz;
              rw[32] = fmaf(t0, __uint_as_float(v[4][j]), ux * px);
              rw[40] = fmaf(t0, __uint_as_float(v[5][j]), uy * py);
              rw[48] = fmaf(t0, __uint_as_float(v[6][j]), uz * pz);
              rw[56] = fmaf(t0, __uint_as_float(v[7][j]), ux * py);
              rw[64] = fmaf(t0, __uint_as_float(v[8][j]), ux * pz);
              rw[72] = fmaf(t0, __uint_as_float(v[9][j]), uy * pz);
            }
            __syncwarp();
            for (int col = lane; col < 80; col += 32) {
              // pairwise: 4 interleaved partial sums of 8 rows, then a tree
              float s4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
              for (int rr = 0; rr < 32; rr++) s4[rr & 3] += red[rr * K::RED + col];
              part[ch * 80 + col] = (s4[0] + s4[1]) + (s4[2] + s4[3]);
            }
            __syncwarp();
          }
        } else {
          for (int i = lane; i < 320; i += 32) part[i] = 0.f;
        }
        ptx::tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          ptx::mbar_arrive(&s.bar[K::B_ACCEMPTY]);
          ptx::mbar_arrive(&s.bar[K::B_EPIFULL + pb]);
        }
      }
      __syncwarp();
      if (ok && lane == 0) ptx::mbar_arrive(&s.bar[K::B_TFREE + par]);
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == K::W_MMA) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, K::TMEM_COLS);
  }
}

// Scratch of the no-allocation NCI entry: the FP64 re-check list (one slot
// per grid point, kNoAllocMaxPoints points at most) followed by its
// counter.  Lives in the module's static device memory, so the entry needs
// no allocation at call time; it is shared by every call on the device.
constexpr int kNoAllocMaxPoints = 1 << 20;
constexpr int kNoAllocTail = 64;  // counter + padding (256 bytes)
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocMaxPoints + kNoAllocTail];

// Nucleus rule on a split-precision grid, located on the device: grid
// points within 1e-5 bohr of a nucleus get s = 0 (src/fieldmod@proc.f90:
// 1148-1154; the same test, d^2 <= 1e-10, as the FP64 NCI sink).  One
// thread per atom; inv is the inverse of xmat (column-major), so a ball of
// radius 1e-5 around the nucleus spans fractional index c within
// 1e-5 * |row c of inv|.  Every grid point in that index box is tested (at
// most 8 per axis: exact for grid steps above 2.5e-6 bohr).  Grid points are
// taken as given, not wrapped into the molecular cell: the same for grids
// inside the cell, which is where critic2's NCI grids lie for molecules.
__global__ void k_nucleus_cgrad(const double4 *atoms, int natom, GridSpec g, Mat3 inv, double *cgrad) {
  const int at = blockIdx.x * blockDim.x + threadIdx.x;
  if (at >= natom) return;
  const double4 A = atoms[at];
  const double r[3] = {A.x - g.x0[0], A.y - g.x0[1], A.z - g.x0[2]};
  long lo[3], hi[3];
  for (int c = 0; c < 3; c++) {
    const double f = inv.m[c] * r[0] + inv.m[3 + c] * r[1] + inv.m[6 + c] * r[2];
    const double rc = 1e-5 * sqrt(inv.m[c] * inv.m[c] + inv.m[3 + c] * inv.m[3 + c] + inv.m[6 + c] * inv.m[6 + c]);
    const double fl = ceil(f - rc), fh = floor(f + rc);
    if (!(fh >= 0.0) || !(fl <= (double)(g.nstep[c] - 1)) || fh < fl) return;
    lo[c] = (long)fmax(fl, 0.0);
    hi[c] = min((long)fmin(fh, (double)(g.nstep[c] - 1)), lo[c] + 7);
  }
  const double xyz[3] = {A.x, A.y, A.z};
  for (long i = lo[0]; i <= hi[0]; i++)
    for (long j = lo[1]; j <= hi[1]; j++)
      for (long k = lo[2]; k <= hi[2]; k++) {
        double d2 = 0.0;
        for (int c = 0; c < 3; c++) {
          const double x = g.x0[c] + i * g.xmat[c] + j * g.xmat[3 + c] + k * g.xmat[6 + c];
          d2 += (x - xyz[c]) * (x - xyz[c]);
        }
        if (d2 <= 1e-10) cgrad[(i * g.nstep[1] + j) * g.nstep[2] + k] = 0.0;
      }
}

// ------------------------------------------------------------------- host
uint32_t morton3(const double *p, const double *lo, const double *span) {
  uint32_t q[3];
  for (int c = 0; c < 3; c++) {
    double f = (p[c] - lo[c]) / (span[c] > 0 ? span[c] : 1.0);
    q[c] = (uint32_t)std::min(1023.0, std::max(0.0, f * 1023.0));
  }
  uint32_t m = 0;
  for (int b = 0; b < 10; b++)
    for (int c = 0; c < 3; c++) m |= ((q[c] >> b) & 1u) << (3 * b + c);
  return m;
}

template <class T>
T *dev_upload(TcOperands *t, const std::vector<T> &v) {
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(1, v.size() * sizeof(T))) != cudaSuccess)
    fail(C2G_ERR_ALLOC, "cudaMalloc (split operands)");
  t->allocs.push_back(p);
  if (!v.empty()) C2G_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return static_cast<T *>(p);
}

uint16_t bf16_bits(float x) {
  const __nv_bfloat16 b = __float2bfloat16_rn(x);
  uint16_t u;
  std::memcpy(&u, &b, 2);
  return u;
}

float bf16_val(uint16_t u) {
  uint32_t w = (uint32_t)u << 16;
  float f;
  std::memcpy(&f, &w, 4);
  return f;
}

// round to nearest (ties away) at the TF32 precision (10 explicit bits)
uint32_t tf32_bits_host(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return u;
  u += 0x1000u;
  return u & 0xffffe000u;
}

float from_bits(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

void ensure_kind(Handle &h, int kind) {
  TcOperands *t = h.tc;
  TcKind &kd = t->kind[kind];
  if (kd.built) return;
  const HostWfn &w = h.host;
  kd.kps = kind == 0 ? 16 : 8;
  kd.nstage = (w.npri + kd.kps - 1) / kd.kps;
  kd.kpad = kd.nstage * kd.kps;
  const int n = (int)t->order.size();
  std::vector<PrimTC> prim(kd.kpad);
  for (int k = 0; k < kd.kpad; k++) {
    if (k < n) {
      const int ip = t->order[k];
      const int *l = kLi[w.itype[ip] - 1];
      prim[k] = PrimTC{};
      prim[k].alpha = (float)w.e[ip];
      prim[k].alpha_lo = (float)(w.e[ip] - (double)prim[k].alpha);
      prim[k].al2e = (float)(w.e[ip] * 1.4426950408889634);
      prim[k].dran = (float)w.dran[ip];
      prim[k].meta = (w.icenter[ip] << 12) | l[0] | (l[1] << 4) | (l[2] << 8);
    } else {
      prim[k] = PrimTC{};  // dran 0: never in range; zero coefficients
      prim[k].alpha = 1.f;
      prim[k].al2e = 1.f;
    }
  }
  const size_t ne = (size_t)t->mo_pad * kd.kpad;
  if (kind == 0) {
    std::vector<uint16_t> hi(ne, 0), lo(ne, 0);
    for (int m = 0; m < w.nmo; m++)
      for (int k = 0; k < n; k++) {
        const double c = w.cmo[(size_t)t->order[k] * w.nmo + m];
        const uint16_t hb = bf16_bits((float)c);
        hi[(size_t)m * kd.kpad + k] = hb;
        lo[(size_t)m * kd.kpad + k] = bf16_bits((float)(c - (double)bf16_val(hb)));
      }
    kd.c_hi = reinterpret_cast<uint8_t *>(dev_upload(t, hi));
    kd.c_lo = reinterpret_cast<uint8_t *>(dev_upload(t, lo));
  } else {
    std::vector<uint32_t> hi(ne, 0), lo(ne, 0);
    for (int m = 0; m < w.nmo; m++)
      for (int k = 0; k < n; k++) {
        const double c = w.cmo[(size_t)t->order[k] * w.nmo + m];
        const uint32_t hb = tf32_bits_host((float)c);
        hi[(size_t)m * kd.kpad + k] = hb;
        lo[(size_t)m * kd.kpad + k] = tf32_bits_host((float)(c - (double)from_bits(hb)));
      }
    kd.c_hi = reinterpret_cast<uint8_t *>(dev_upload(t, hi));
    kd.c_lo = reinterpret_cast<uint8_t *>(dev_upload(t, lo));
  }
  kd.prim = dev_upload(t, prim);
  std::vector<int> soff(kd.nstage + 1, 0);
  std::vector<float4> sent;
  for (int st = 0; st < kd.nstage; st++) {
    soff[st] = (int)sent.size();
    const size_t first = sent.size();
    for (int k = st * kd.kps; k < (st + 1) * kd.kps && k < n; k++) {
      const int at = prim[k].meta >> 12;
      if (!(prim[k].dran > 0.f)) continue;
      size_t e = first;
      while (e < sent.size() && std::memcmp(&sent[e].x, &at, 4) != 0) e++;
      if (e == sent.size()) {
        float4 E;
        std::memcpy(&E.x, &at, 4);
        E.y = prim[k].dran;
        E.z = prim[k].alpha;
        E.w = 0.f;
        sent.push_back(E);
      } else {
        sent[e].y = std::max(sent[e].y, prim[k].dran);
        sent[e].z = std::min(sent[e].z, prim[k].alpha);
      }
    }
  }
  soff[kd.nstage] = (int)sent.size();
  kd.soff = dev_upload(t, soff);
  kd.sent = dev_upload(t, sent);
  kd.built = true;
}

int kind_of(int prec) {
  if (prec == C2G_PREC_BF16X3) return 0;
  if (prec == C2G_PREC_TF32X3) return 1;
  fail(C2G_ERR_ARG, "not a split-precision mode");
}

TcArgs make_args(Handle &h, int kind) {
  ensure_kind(h, kind);
  TcOperands *t = h.tc;
  const TcKind &kd = t->kind[kind];
  TcArgs a{};
  a.w = h.dev;
  a.prim = kd.prim;
  a.soff = kd.soff;
  a.sent = kd.sent;
  a.c_hi = kd.c_hi;
  a.c_lo = kd.c_lo;
  a.occ = t->occ;
  a.nstage = kd.nstage;
  a.kpad = kd.kpad;
  a.nmt = t->nmt;
  a.maskw = (kd.nstage + 31) / 32;
  a.err = t->err;
  a.recheck = nullptr;
  a.recheck_count = nullptr;
  a.recheck_cap = 0;
  // Split Hessians carry ~1e-6 (TF32x3) / ~2e-5 (BF16x3) relative error, so
  // sign(lambda2) can only be wrong well below these thresholds.
  a.recheck_rel = (float)(t->recheck_rel >= 0.0 ? t->recheck_rel : (kind == 1 ? 1e-4 : 1e-3));
  a.stage_count = nullptr;
  a.wait_ns = t->wait_ns;
  return a;
}

int sm_count() {
  int dev = 0, n = 0;
  C2G_CUDA(cudaGetDevice(&dev));
  C2G_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  return n;
}

constexpr size_t kSmemLimit = 227 * 1024;

// Shared memory of a launch; whether the per-tile atom tables fit in it.
size_t tc_smem(const TcArgs &a, bool &atoms_smem) {
  size_t offs[15];
  size_t bytes = smem_bytes(a.w.natom, a.maskw, true, offs);
  atoms_smem = bytes <= kSmemLimit;
  if (!atoms_smem) bytes = smem_bytes(a.w.natom, a.maskw, false, offs);
  if (bytes > kSmemLimit)
    fail(C2G_ERR_UNSUPPORTED, "too many primitives for the split-precision kernel's shared memory");
  return bytes;
}

template <int KIND, class Src, class Sink>
void launch_tc(const TcArgs &a, const Src &src, const Sink &sink, int ntiles, int grid, size_t bytes,
               cudaStream_t st) {
  auto fn = k_tc<KIND, Src, Sink>;
  C2G_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  fn<<<grid, K::NTHR, bytes, st>>>(a, src, sink, ntiles);
  C2G_CUDA(cudaGetLastError());
}

// Launches the split kernel over ntiles 32-point tiles, one CTA per SM at
// most.  Molecules whose per-tile atom tables do not fit shared memory get
// them in a per-CTA slice of a global buffer owned by the handle (grown on
// demand); with allow_alloc false (the no-allocation entry) such molecules
// are refused.
template <class Src, class Sink>
void launch_kind(Handle &h, int kind, TcArgs a, const Src &src, const Sink &sink, int ntiles, cudaStream_t st,
                 bool allow_alloc = true) {
  if (ntiles <= 0) return;
  const int grid = std::min(ntiles, sm_count());
  bool atoms_smem = true;
  a.atab = nullptr;
  a.atab_stride = atom_table_bytes(a.w.natom);
  tc_smem(a, atoms_smem);
  if (!atoms_smem) {
    if (!allow_alloc)
      fail(C2G_ERR_UNSUPPORTED, "molecule too large for the no-allocation entry (" + std::to_string(a.w.natom) +
                                    " atoms: the per-tile atom tables do not fit shared memory)");
    TcOperands *t = h.tc;
    const size_t need = a.atab_stride * (size_t)grid;
    if (t->atab_cap < need) {
      if (t->atab) cudaFree(t->atab);
      t->atab = nullptr;
      t->atab_cap = 0;
      if (cudaMalloc(&t->atab, need) != cudaSuccess) fail(C2G_ERR_ALLOC, "cudaMalloc (atom tables)");
      t->atab_cap = need;
    }
    a.atab = t->atab;
  }
  const size_t bytes = tc_smem(a, atoms_smem);
  if (kind == 0) launch_tc<0>(a, src, sink, ntiles, grid, bytes, st);
  else launch_tc<1>(a, src, sink, ntiles, grid, bytes, st);
}

void check_device_error(TcOperands *t) {
  int e = 0;
  C2G_CUDA(cudaMemcpy(&e, t->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    C2G_CUDA(cudaMemset(t->err, 0, sizeof(int)));
    fail(C2G_ERR_CUDA, "split-precision kernel: a pipeline wait timed out (mask " + std::to_string(e) + ")");
  }
}

// Launches the nucleus rule for a grid on the stream (nothing when xmat is
// singular or the molecule has no atoms).
void launch_nucleus_rule(const Handle &h, const GridSpec &g, double *d_cgrad, cudaStream_t st) {
  const double *M = g.xmat;
  const double det = M[0] * (M[4] * M[8] - M[7] * M[5]) - M[3] * (M[1] * M[8] - M[7] * M[2]) +
                     M[6] * (M[1] * M[5] - M[4] * M[2]);
  if (det == 0.0 || h.dev.natom <= 0) return;
  Mat3 inv;
  inv.m[0] = (M[4] * M[8] - M[5] * M[7]) / det;
  inv.m[3] = (M[5] * M[6] - M[3] * M[8]) / det;
  inv.m[6] = (M[3] * M[7] - M[4] * M[6]) / det;
  inv.m[1] = (M[2] * M[7] - M[1] * M[8]) / det;
  inv.m[4] = (M[0] * M[8] - M[2] * M[6]) / det;
  inv.m[7] = (M[1] * M[6] - M[0] * M[7]) / det;
  inv.m[2] = (M[1] * M[5] - M[2] * M[4]) / det;
  inv.m[5] = (M[2] * M[3] - M[0] * M[5]) / det;
  inv.m[8] = (M[0] * M[4] - M[1] * M[3]) / det;
  k_nucleus_cgrad<<<(h.dev.natom + 127) / 128, 128, 0, st>>>(h.dev.atoms, h.dev.natom, g, inv, d_cgrad);
  C2G_CUDA(cudaGetLastError());
}

}  // namespace

TcOperands *tc_create(Handle &h) {
  auto *t = new TcOperands();
  try {
    const HostWfn &w = h.host;
    t->mo_pad = (w.nmo + K::MT - 1) / K::MT * K::MT;
    t->nmt = t->mo_pad / K::MT;
    // Primitive order for the K-stages: diffuse to compact by cutoff
    // bucket (factors of 2), then by the atom's Morton code, keeping each
    // atom's primitives (and so each shell) together.
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < w.natom; a++)
      for (int c = 0; c < 3; c++) lo[c] = std::min(lo[c], w.xyz[3 * a + c]), hi[c] = std::max(hi[c], w.xyz[3 * a + c]);
    const double span[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    std::vector<uint32_t> mort(w.natom);
    for (int a = 0; a < w.natom; a++) mort[a] = morton3(&w.xyz[3 * a], lo, span);
    t->order.resize(w.npri);
    std::iota(t->order.begin(), t->order.end(), 0);
    auto bucket = [&](int ip) { return -(int)std::floor(std::log2(w.dran[ip])); };
    std::stable_sort(t->order.begin(), t->order.end(), [&](int x, int y) {
      const int bx = bucket(x), by = bucket(y);
      if (bx != by) return bx < by;
      const int ax = w.icenter[x], ay = w.icenter[y];
      if (mort[ax] != mort[ay]) return mort[ax] < mort[ay];
      return ax < ay;
    });
    std::vector<float> occ(t->mo_pad, 0.f);
    for (int m = 0; m < w.nmo; m++) occ[m] = (float)w.occ[m];
    t->occ = dev_upload(t, occ);
    std::vector<int> zero(1, 0);
    t->err = dev_upload(t, zero);
  } catch (...) {
    tc_destroy(t);
    throw;
  }
  return t;
}

void tc_destroy(TcOperands *t) {
  if (!t) return;
  for (void *p : t->allocs) cudaFree(p);
  if (t->scratch) cudaFree(t->scratch);
  if (t->atab) cudaFree(t->atab);
  delete t;
}

void tc_set_recheck(Handle &h, double rel) { h.tc->recheck_rel = rel; }

void tc_set_wait_ns(Handle &h, uint64_t ns) { h.tc->wait_ns = ns; }

void tc_check_error(Handle &h) { check_device_error(h.tc); }

void tc_points(Handle &h, int prec, int n, const double *d_xyz, double *d_rec, cudaStream_t st, bool wrap) {
  const int kind = kind_of(prec);
  TcArgs a = make_args(h, kind);
  ListSrc src{d_xyz, n, wrap};
  launch_kind(h, kind, a, src, TcRecSink{d_rec}, (n + 31) / 32, st);
  C2G_CUDA(cudaStreamSynchronize(st));
  check_device_error(h.tc);
}

void tc_points_index(Handle &h, int prec, const double *d_x, const int *d_idx, const int *d_count, int maxn,
                     double *d_rec, cudaStream_t st) {
  const int kind = kind_of(prec);
  TcArgs a = make_args(h, kind);
  IndexSrc src{d_x, d_idx, d_count};
  launch_kind(h, kind, a, src, TcRecSink{d_rec}, (maxn + 31) / 32, st);
}

long tc_nci_grid(Handle &h, int prec, const GridSpec &g, double *d_crho, double *d_cgrad, cudaStream_t st,
                 cudaEvent_t ev_split, double *stage_frac) {
  const int kind = kind_of(prec);
  TcArgs a = make_args(h, kind);
  const long npts = (long)g.nstep[0] * g.nstep[1] * g.nstep[2];
  // scratch: re-check list (one slot per point) and its counter
  TcOperands *t = h.tc;
  if (t->scratch_cap < (size_t)npts + 8) {
    if (t->scratch) cudaFree(t->scratch);
    t->scratch = nullptr;
    t->scratch_cap = 0;
    if (cudaMalloc(&t->scratch, sizeof(int) * ((size_t)npts + 8)) != cudaSuccess)
      fail(C2G_ERR_ALLOC, "cudaMalloc (re-check list)");
    t->scratch_cap = (size_t)npts + 8;
  }
  int *scratch = t->scratch;
  int *count = scratch + npts;
  // the 64-bit stage counter sits at an 8-byte aligned slot after the count
  unsigned long long *stage_count = reinterpret_cast<unsigned long long *>(scratch + ((npts + 2) & ~1L) + 2);
  C2G_CUDA(cudaMemsetAsync(count, 0, sizeof(int) * 8, st));
  a.stage_count = stage_count;
  a.recheck = scratch;
  a.recheck_count = count;
  a.recheck_cap = (int)npts;
  GridSrc src{g, (g.nstep[1] + 3) / 4, (g.nstep[2] + 7) / 8};
  const long ntiles = (long)g.nstep[0] * src.ntj * src.ntk;
  launch_kind(h, kind, a, src, TcNciSink{d_crho, d_cgrad}, (int)ntiles, st);
  if (ev_split) C2G_CUDA(cudaEventRecord(ev_split, st));
  // FP64 re-evaluation of the listed points (the count is read on device)
  launch_fp64_nci_list(h.dev, g, scratch, count, (int)npts, d_crho, d_cgrad, st);
  // nucleus rule: |grad| := 0 (s = 0) at grid points within 1e-5 bohr of a nucleus
  launch_nucleus_rule(h, g, d_cgrad, st);
  int hcount = 0;
  unsigned long long hstages = 0;
  C2G_CUDA(cudaMemcpyAsync(&hcount, count, sizeof(int), cudaMemcpyDeviceToHost, st));
  C2G_CUDA(cudaMemcpyAsync(&hstages, stage_count, sizeof(hstages), cudaMemcpyDeviceToHost, st));
  C2G_CUDA(cudaStreamSynchronize(st));
  check_device_error(h.tc);
  if (stage_frac) *stage_frac = (double)hstages / ((double)ntiles * t->kind[kind].nstage);
  return hcount;
}

long tc_noalloc_max_points() { return kNoAllocMaxPoints; }

void tc_nci_grid_noalloc(Handle &h, int prec, const GridSpec &g, double *d_crho, double *d_cgrad, cudaStream_t st) {
  const int kind = kind_of(prec);
  TcOperands *t = h.tc;
  if (!t->kind[kind].built)
    fail(C2G_ERR_UNSUPPORTED,
         "the split operands of this precision mode are not on the device yet; they are allocated by the first "
         "split-precision call of an allocating entry (e.g. c2g_nciplot_dev on a 1-point grid)");
  const long npts = (long)g.nstep[0] * g.nstep[1] * g.nstep[2];
  if (npts > kNoAllocMaxPoints)
    fail(C2G_ERR_ARG, "grid has " + std::to_string(npts) + " points; the no-allocation entry takes at most " +
                          std::to_string(kNoAllocMaxPoints) + " per call (split the grid into slabs)");
  // once per device, with that device current: the address of the scratch
  static std::mutex mu;
  static int *ptr_of[64] = {nullptr};
  int dev = 0;
  C2G_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) fail(C2G_ERR_UNSUPPORTED, "device ordinal above 63");
  int *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!ptr_of[dev]) {
      void *p = nullptr;
      const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (rc != cudaSuccess) fail(C2G_ERR_CUDA, std::string("cudaGetSymbolAddress (no-allocation scratch): ") +
                                                    cudaGetErrorString(rc));
      ptr_of[dev] = static_cast<int *>(p);
    }
    scratch = ptr_of[dev];
  }
  int *count = scratch + kNoAllocMaxPoints;
  // the re-check counter must start at zero
  C2G_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
  TcArgs a = make_args(h, kind);
  a.recheck = scratch;
  a.recheck_count = count;
  a.recheck_cap = (int)npts;
  GridSrc src{g, (g.nstep[1] + 3) / 4, (g.nstep[2] + 7) / 8};
  const long ntiles = (long)g.nstep[0] * src.ntj * src.ntk;
  launch_kind(h, kind, a, src, TcNciSink{d_crho, d_cgrad}, (int)ntiles, st, false);
  launch_fp64_nci_list(h.dev, g, scratch, count, (int)npts, d_crho, d_cgrad, st);
  launch_nucleus_rule(h, g, d_cgrad, st);
  // pipeline timeouts of the split kernel are reported by this call
  int e = 0;
  C2G_CUDA(cudaMemcpyAsync(&e, t->err, sizeof(int), cudaMemcpyDeviceToHost, st));
  C2G_CUDA(cudaStreamSynchronize(st));
  if (e) {
    C2G_CUDA(cudaMemsetAsync(t->err, 0, sizeof(int), st));
    C2G_CUDA(cudaStreamSynchronize(st));
    fail(C2G_ERR_CUDA, "split-precision kernel: a pipeline wait timed out (mask " + std::to_string(e) + ")");
  }
}

}  // namespace c2g
