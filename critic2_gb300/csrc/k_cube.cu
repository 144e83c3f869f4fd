// NCI post-pass and text output on the GPU: critic2's cutoff pass over the
// grid (src/nci@proc.f90:612-645) and its cube/dat writers
// (src/nci@proc.f90:818-932, the .dat lines of :637-639).
//
// The post-pass flags the points that go to the .dat file (|crho| <
// rhocut*100 and s < dimcut), compacts their (crho/100, s) pairs in grid
// order, and then sets s := 100 where |crho| > rhoplot*100, outside
// srhorange, or (onlyneg) where crho > 0, exactly as the reference does.
//
// Text is formatted on the device, one thread per number: the Fortran
// edit descriptors 1p,e13.5e3 (cube bodies, 6 numbers per line, one record
// per (i,j) row) and 1p,E15.7 (dat lines).  The decimal digits come from
// x * 10^s in FP64; a number whose scaled value lies within a small margin
// of a rounding boundary (1e-7 of a unit in the last digit) is listed, and
// the host rewrites exactly those with the C library's correctly rounded
// conversion, so the text is the correctly rounded decimal of every value.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "c2g_internal.h"
#include "k_cube.h"
#include "k_tc.h"

namespace c2g {

// ------------------------------------------------------- host formatting
// Fortran 1p,e13.5e3 with the leading blank of the (" ",...) edit list:
// 14 characters, e.g. " -6.92253E+000".
void fmt_e13_5e3(double x, char *out) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%.5E", x);  // [-]d.dddddE[+-]dd[d]
  const char *p = std::strchr(buf, 'E');
  const int e = std::atoi(p + 1);
  const int ml = (int)(p - buf);  // mantissa length incl. sign
  char t[16];
  int k = 0;
  t[k++] = ' ';
  if (buf[0] != '-') t[k++] = ' ';
  for (int i = 0; i < ml; i++) t[k++] = buf[i];
  t[k++] = 'E';
  t[k++] = e < 0 ? '-' : '+';
  const int ae = e < 0 ? -e : e;
  t[k++] = (char)('0' + ae / 100);
  t[k++] = (char)('0' + (ae / 10) % 10);
  t[k++] = (char)('0' + ae % 10);
  std::memcpy(out, t, 14);
}

// Fortran 1p,E15.7: 15 characters; exponents beyond +-99 lose the 'E'.
void fmt_E15_7(double x, char *out) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%.7E", x);
  const char *p = std::strchr(buf, 'E');
  const int e = std::atoi(p + 1);
  const int ml = (int)(p - buf);
  char t[24];
  int k = 0;
  const int ae = e < 0 ? -e : e;
  for (int i = 0; i < 15 - (ml + 4); i++) t[k++] = ' ';  // the exponent field is 4 wide
  for (int i = 0; i < ml; i++) t[k++] = buf[i];
  if (ae > 99) {
    t[k++] = e < 0 ? '-' : '+';
    t[k++] = (char)('0' + ae / 100);
    t[k++] = (char)('0' + (ae / 10) % 10);
    t[k++] = (char)('0' + ae % 10);
  } else {
    t[k++] = 'E';
    t[k++] = e < 0 ? '-' : '+';
    t[k++] = (char)('0' + ae / 10);
    t[k++] = (char)('0' + ae % 10);
  }
  std::memcpy(out, t, 15);
}

// A record of n3 numbers: 14 characters each, a newline after every 6th
// and after the last, and one blank before that last newline when the line
// holds fewer than 6 (Fortran writes the (" ") of the next item before it
// finds the list exhausted).
// Fortran E22.14E3 (no scale factor): 0.dddddddddddddd with 14 digits and
// a 3-digit exponent, right-justified in 22 columns.
void fmt_E22_14E3(double x, char *out) {
  char buf[48];
  std::snprintf(buf, sizeof buf, "%.13E", x);  // [-]d.dddddddddddddE[+-]dd[d]
  const char *p = std::strchr(buf, 'E');
  const int e = std::atoi(p + 1) + (x != 0.0 ? 1 : 0);
  const bool neg = buf[0] == '-';
  const char *m = buf + (neg ? 1 : 0);  // d.ddddddddddddd
  char t[24];
  t[0] = neg ? '-' : ' ';
  t[1] = '0';
  t[2] = '.';
  t[3] = m[0];
  for (int i = 0; i < 13; i++) t[4 + i] = m[2 + i];
  t[17] = 'E';
  t[18] = e < 0 ? '-' : '+';
  const int ae = e < 0 ? -e : e;
  t[19] = (char)('0' + ae / 100);
  t[20] = (char)('0' + (ae / 10) % 10);
  t[21] = (char)('0' + ae % 10);
  std::memcpy(out, t, 22);
}

long precise_record_bytes(int n3) { return 23L * n3 + (n3 + 5) / 6 + (n3 % 6 ? 1 : 0); }

long precise_body_bytes(const int *n) { return precise_record_bytes(n[2]) * n[0] * n[1]; }

long cube_record_bytes(int n3) { return 14L * n3 + (n3 + 5) / 6 + (n3 % 6 ? 1 : 0); }

long cube_body_bytes(const int *n) { return cube_record_bytes(n[2]) * n[0] * n[1]; }

namespace {

constexpr int kFlagCap = 1 << 16;

// ------------------------------------------------------ device formatting
__device__ __forceinline__ double scale10(double a, int s) {
  // a * 10^s, exact powers of ten up to 10^22 per step
  const double p22 = 1e22;
  while (s > 22) a *= p22, s -= 22;
  while (s < -22) a /= p22, s += 22;
  double p = 1.0;
  for (int i = 0; i < (s < 0 ? -s : s); i++) p *= 10.0;  // exact for |s| <= 22
  return s >= 0 ? a * p : a / p;
}

// D significant digits of a > 0: n in [10^(D-1), 10^D), a ~ n 10^(e-D+1).
// Returns false when the scaled value is within `margin` of a rounding
// boundary (the host then formats the number).
__device__ bool dec_digits(double a, int D, double margin, long long &n, int &e) {
  double lo = 1.0;
  for (int i = 1; i < D; i++) lo *= 10.0;
  const double hi = lo * 10.0;
  int e0 = (int)floor(log10(a));
  for (int it = 0; it < 4; it++) {
    const double y = scale10(a, D - 1 - e0);
    const double r = rint(y);
    if (r >= hi) {
      e0++;
      continue;
    }
    if (r < lo) {
      e0--;
      continue;
    }
    n = (long long)r;
    e = e0;
    const double f = y - floor(y);
    return fabs(f - 0.5) > margin;
  }
  return false;
}

__device__ __forceinline__ void put_digits(char *o, long long n, int D) {
  // d.ddd..: D digits with a point after the first
  for (int i = D; i >= 2; i--) {
    o[i] = (char)('0' + (int)(n % 10));
    n /= 10;
  }
  o[1] = '.';
  o[0] = (char)('0' + (int)n);
}

// 14 characters of " " + 1p,e13.5e3; returns false for a near tie
__device__ bool dev_e13(double x, char *o) {
  const bool neg = signbit(x);
  const double a = fabs(x);
  long long n = 0;
  int e = 0;
  bool ok = true;
  if (a == 0.0) {
    n = 100000;
    e = 0;
  } else {
    ok = dec_digits(a, 6, 1e-7, n, e);
  }
  char t[14];
  t[0] = ' ';
  t[1] = neg ? '-' : ' ';
  put_digits(t + 2, a == 0.0 ? 0 : n, 6);
  t[9] = 'E';
  t[10] = e < 0 ? '-' : '+';
  const int ae = e < 0 ? -e : e;
  t[11] = (char)('0' + ae / 100);
  t[12] = (char)('0' + (ae / 10) % 10);
  t[13] = (char)('0' + ae % 10);
  for (int i = 0; i < 14; i++) o[i] = t[i];
  return ok;
}

// 15 characters of 1p,E15.7; returns false for a near tie
__device__ bool dev_E15(double x, char *o) {
  const bool neg = signbit(x);
  const double a = fabs(x);
  long long n = 0;
  int e = 0;
  bool ok = true;
  if (a == 0.0) {
    n = 0;
    e = 0;
  } else {
    ok = dec_digits(a, 8, 1e-6, n, e);
  }
  char t[15];
  t[0] = ' ';
  t[1] = neg ? '-' : ' ';
  put_digits(t + 2, n, 8);
  const int ae = e < 0 ? -e : e;
  if (ae > 99) {
    // three-digit exponents: Fortran writes sign and digits without the E
    t[11] = e < 0 ? '-' : '+';
    t[12] = (char)('0' + ae / 100);
    t[13] = (char)('0' + (ae / 10) % 10);
    t[14] = (char)('0' + ae % 10);
  } else {
    t[11] = 'E';
    t[12] = e < 0 ? '-' : '+';
    t[13] = (char)('0' + ae / 10);
    t[14] = (char)('0' + ae % 10);
  }
  for (int i = 0; i < 15; i++) o[i] = t[i];
  return ok;
}

// a * 10^s as a double-double hi + lo (error ~1e-30 relative): exact
// products with the exact powers 10^0..10^22, exact remainders for
// divisions.
__device__ __forceinline__ void dd_scale10(double a, int s, double &hi, double &lo) {
  hi = a;
  lo = 0.0;
  while (s != 0) {
    const int k = s > 22 ? 22 : (s < -22 ? -22 : s);
    double p = 1.0;
    for (int i = 0; i < (k < 0 ? -k : k); i++) p *= 10.0;
    if (k > 0) {
      const double h = hi * p;
      const double e = fma(hi, p, -h);
      hi = h;
      lo = fma(lo, p, e);
    } else {
      const double q = hi / p;
      const double r = fma(-q, p, hi);  // exact remainder
      hi = q;
      lo = (r + lo) / p;
    }
    // renormalise
    const double t = hi + lo;
    lo = lo - (t - hi);
    hi = t;
    s -= k;
  }
}

// D significant digits (D <= 15) of a > 0 from the double-double product;
// false when within `margin` of a rounding boundary.
__device__ bool dd_digits(double a, int D, double margin, long long &n, int &e) {
  double lo10 = 1.0;
  for (int i = 1; i < D; i++) lo10 *= 10.0;
  const double hi10 = lo10 * 10.0;
  int e0 = (int)floor(log10(a));
  for (int it = 0; it < 4; it++) {
    double yh, yl;
    dd_scale10(a, D - 1 - e0, yh, yl);
    double r = rint(yh);
    double f = (yh - r) + yl;  // in about [-0.5, 0.5]
    if (f > 0.5) r += 1.0, f -= 1.0;
    if (f <= -0.5) r -= 1.0, f += 1.0;
    if (r >= hi10) {
      e0++;
      continue;
    }
    if (r < lo10) {
      e0--;
      continue;
    }
    n = (long long)r;
    e = e0;
    return fabs(fabs(f) - 0.5) > margin;
  }
  return false;
}

// 23 characters of " " + E22.14E3; false for a near tie
__device__ bool dev_E22(double x, char *o) {
  const bool neg = signbit(x);
  const double a = fabs(x);
  long long n = 0;
  int e = 0;
  bool ok = true;
  if (a != 0.0) ok = dd_digits(a, 14, 1e-6, n, e), e += 1;
  char t[23];
  t[0] = ' ';
  t[1] = neg ? '-' : ' ';
  t[2] = '0';
  t[3] = '.';
  for (int i = 17; i >= 4; i--) {
    t[i] = (char)('0' + (int)(n % 10));
    n /= 10;
  }
  t[18] = 'E';
  t[19] = e < 0 ? '-' : '+';
  const int ae = e < 0 ? -e : e;
  t[20] = (char)('0' + ae / 100);
  t[21] = (char)('0' + (ae / 10) % 10);
  t[22] = (char)('0' + ae % 10);
  for (int i = 0; i < 23; i++) o[i] = t[i];
  return ok;
}

__global__ void k_precise_text(const double *__restrict__ v, long n, int n3, long rec_bytes,
                               char *__restrict__ text, int *__restrict__ flags, int *__restrict__ nflag) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long rec = i / n3;
  const int m = (int)(i - rec * n3);
  char *o = text + rec * rec_bytes + 23L * m + m / 6;
  if (!dev_E22(v[i], o)) {
    const int s = atomicAdd(nflag, 1);
    if (s < kFlagCap) flags[s] = (int)i;
  }
  if (m == n3 - 1 && n3 % 6 != 0) {
    o[23] = ' ';
    o[24] = '\n';
  } else if (m % 6 == 5) {
    o[23] = '\n';
  }
}

__global__ void k_cube_text(const double *__restrict__ v, long n, int n3, long rec_bytes, char *__restrict__ text,
                            int *__restrict__ flags, int *__restrict__ nflag) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long rec = i / n3;
  const int m = (int)(i - rec * n3);
  char *o = text + rec * rec_bytes + 14L * m + m / 6;
  if (!dev_e13(v[i], o)) {
    const int s = atomicAdd(nflag, 1);
    if (s < kFlagCap) flags[s] = (int)i;
  }
  if (m == n3 - 1 && n3 % 6 != 0) {
    o[14] = ' ';
    o[15] = '\n';
  } else if (m % 6 == 5) {
    o[14] = '\n';
  }
}

__global__ void k_dat_text(const double *__restrict__ d, long n, char *__restrict__ text, int *__restrict__ flags,
                           int *__restrict__ nflag) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 2 * n) return;
  const long line = i >> 1;
  const int f = (int)(i & 1);
  char *o = text + line * 31 + 15 * f;
  if (!dev_E15(d[i], o)) {
    const int s = atomicAdd(nflag, 1);
    if (s < kFlagCap) flags[s] = (int)i;
  }
  if (f) o[15] = '\n';
}

// ------------------------------------------------------------ post-pass
__device__ __forceinline__ bool in_dat(double cr, double cg, const NciCut &c) {
  return fabs(cr) < c.rhocut * 100.0 && cg < c.dimcut;
}

__global__ void k_post_count(const double *__restrict__ crho, const double *__restrict__ cgrad, long n, NciCut c,
                             int *__restrict__ bcount) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = i < n && in_dat(crho[i], cgrad[i], c);
  const int cnt = __syncthreads_count(f);
  if (threadIdx.x == 0) bcount[blockIdx.x] = cnt;
}

// exclusive scan of the block counts by one block (nb may be large)
__global__ void k_scan(int *__restrict__ bcount, int nb, long *__restrict__ total) {
  __shared__ long s_carry;
  __shared__ int s_w[32];
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    const int v = b < nb ? bcount[b] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[wp] = x;
    __syncthreads();
    if (wp == 0) {
      int w = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      s_w[lane] = w;
    }
    __syncthreads();
    const long base = s_carry + (wp > 0 ? s_w[wp - 1] : 0);
    if (b < nb) bcount[b] = (int)(base + x - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = base + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = s_carry;
}

__global__ void k_post_apply(const double *__restrict__ crho, double *__restrict__ cgrad, long n, NciCut c,
                             const int *__restrict__ boff, double *__restrict__ dat, long cap) {
  __shared__ int s_w[32];
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  double cr = 0.0, cg = 0.0;
  bool f = false;
  if (i < n) {
    cr = crho[i];
    cg = cgrad[i];
    f = in_dat(cr, cg, c);
  }
  const unsigned b = __ballot_sync(0xffffffffu, f);
  if (lane == 0) s_w[wp] = __popc(b);
  __syncthreads();
  int off = boff[blockIdx.x];
  for (int w = 0; w < wp; w++) off += s_w[w];
  if (f) {
    const long slot = off + __popc(b & ((1u << lane) - 1u));
    if (slot < cap) {
      dat[2 * slot] = cr / 100.0;
      dat[2 * slot + 1] = cg;
    }
  }
  if (i < n) {
    const bool big = fabs(cr) > c.rhoplot * 100.0;
    const bool out = cr < c.srho_lo * 100.0 || cr > c.srho_hi * 100.0;
    const bool neg = c.onlyneg && cr > 0.0;
    if (big || out || neg) cgrad[i] = 100.0;
  }
}

// mode: 0 cube e13.5e3, 1 dat E15.7, 2 cube E22.14E3
void fix_flags(const int *d_flags, const int *d_nflag, const double *d_v, char *text, bool on_device, int mode,
               int n3, long rec_bytes, cudaStream_t st) {
  int nf = 0;
  C2G_CUDA(cudaMemcpyAsync(&nf, d_nflag, sizeof(int), cudaMemcpyDeviceToHost, st));
  C2G_CUDA(cudaStreamSynchronize(st));
  if (nf > kFlagCap) fail(C2G_ERR_UNSUPPORTED, "too many near-tie numbers in one text block");
  if (nf == 0) return;
  std::vector<int> idx(nf);
  C2G_CUDA(cudaMemcpy(idx.data(), d_flags, sizeof(int) * nf, cudaMemcpyDeviceToHost));
  for (int q = 0; q < nf; q++) {
    const long i = idx[q];
    double x = 0.0;
    C2G_CUDA(cudaMemcpy(&x, d_v + i, sizeof(double), cudaMemcpyDeviceToHost));
    char buf[32];
    long off;
    int len;
    if (mode == 0) {
      const long rec = i / n3;
      const int m = (int)(i - rec * n3);
      off = rec * rec_bytes + 14L * m + m / 6;
      fmt_e13_5e3(x, buf);
      len = 14;
    } else if (mode == 2) {
      const long rec = i / n3;
      const int m = (int)(i - rec * n3);
      off = rec * rec_bytes + 23L * m + m / 6 + 1;  // after the separator blank
      fmt_E22_14E3(x, buf);
      len = 22;
    } else {
      off = (i >> 1) * 31 + 15 * (i & 1);
      fmt_E15_7(x, buf);
      len = 15;
    }
    if (on_device) C2G_CUDA(cudaMemcpy(text + off, buf, len, cudaMemcpyHostToDevice));
    else std::memcpy(text + off, buf, len);
  }
}

}  // namespace

void cube_text_dev(const int *nstep, const double *d_v, char *d_text, char *h_text, int *d_scratch,
                   cudaStream_t st) {
  const long n = (long)nstep[0] * nstep[1] * nstep[2];
  const long rb = cube_record_bytes(nstep[2]);
  int *nflag = d_scratch, *flags = d_scratch + 8;
  C2G_CUDA(cudaMemsetAsync(nflag, 0, sizeof(int), st));
  if (n > 0) {
    k_cube_text<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_v, n, nstep[2], rb, d_text, flags, nflag);
    C2G_CUDA(cudaGetLastError());
  }
  if (h_text) {
    C2G_CUDA(cudaMemcpyAsync(h_text, d_text, (size_t)(rb * nstep[0] * nstep[1]), cudaMemcpyDeviceToHost, st));
    fix_flags(flags, nflag, d_v, h_text, false, 0, nstep[2], rb, st);
  } else {
    fix_flags(flags, nflag, d_v, d_text, true, 0, nstep[2], rb, st);
  }
}

void precise_text_dev(const int *nstep, const double *d_v, char *d_text, char *h_text, int *d_scratch,
                      cudaStream_t st) {
  const long n = (long)nstep[0] * nstep[1] * nstep[2];
  const long rb = precise_record_bytes(nstep[2]);
  int *nflag = d_scratch, *flags = d_scratch + 8;
  C2G_CUDA(cudaMemsetAsync(nflag, 0, sizeof(int), st));
  if (n > 0) {
    k_precise_text<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_v, n, nstep[2], rb, d_text, flags, nflag);
    C2G_CUDA(cudaGetLastError());
  }
  if (h_text) {
    C2G_CUDA(cudaMemcpyAsync(h_text, d_text, (size_t)(rb * nstep[0] * nstep[1]), cudaMemcpyDeviceToHost, st));
    fix_flags(flags, nflag, d_v, h_text, false, 2, nstep[2], rb, st);
  } else {
    fix_flags(flags, nflag, d_v, d_text, true, 2, nstep[2], rb, st);
  }
}

void dat_text_dev(const double *d_dat, long ndat, char *d_text, char *h_text, int *d_scratch, cudaStream_t st) {
  int *nflag = d_scratch, *flags = d_scratch + 8;
  C2G_CUDA(cudaMemsetAsync(nflag, 0, sizeof(int), st));
  if (ndat > 0) {
    k_dat_text<<<(unsigned)((2 * ndat + 255) / 256), 256, 0, st>>>(d_dat, ndat, d_text, flags, nflag);
    C2G_CUDA(cudaGetLastError());
  }
  if (h_text) {
    C2G_CUDA(cudaMemcpyAsync(h_text, d_text, (size_t)(31 * ndat), cudaMemcpyDeviceToHost, st));
    fix_flags(flags, nflag, d_dat, h_text, false, 1, 0, 0, st);
  } else {
    fix_flags(flags, nflag, d_dat, d_text, true, 1, 0, 0, st);
  }
}

long nci_post_dev(const int *nstep, const double *d_crho, double *d_cgrad, const NciCut &cut, double *d_dat,
                  long cap, int *d_bcount, long *d_total, cudaStream_t st) {
  const long n = (long)nstep[0] * nstep[1] * nstep[2];
  if (n <= 0) return 0;
  const int nb = (int)((n + 255) / 256);
  k_post_count<<<nb, 256, 0, st>>>(d_crho, d_cgrad, n, cut, d_bcount);
  C2G_CUDA(cudaGetLastError());
  k_scan<<<1, 1024, 0, st>>>(d_bcount, nb, d_total);
  C2G_CUDA(cudaGetLastError());
  k_post_apply<<<nb, 256, 0, st>>>(d_crho, d_cgrad, n, cut, d_bcount, d_dat, cap);
  C2G_CUDA(cudaGetLastError());
  long total = 0;
  C2G_CUDA(cudaMemcpyAsync(&total, d_total, sizeof(long), cudaMemcpyDeviceToHost, st));
  C2G_CUDA(cudaStreamSynchronize(st));
  return total;
}

int cube_flag_scratch_ints() { return 8 + kFlagCap; }

namespace {

// grid points x0 + i xmat(:,1) + j xmat(:,2) + k xmat(:,3), k fastest, for
// the i-planes [i0, i0 + ni)
__global__ void k_grid_points(GridSpec g, int i0, long n, double *__restrict__ xyz) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long plane = (long)g.nstep[1] * g.nstep[2];
  const int i = i0 + (int)(t / plane);
  const long r = t % plane;
  const int j = (int)(r / g.nstep[2]), k = (int)(r % g.nstep[2]);
  for (int c = 0; c < 3; c++) xyz[3 * t + c] = g.x0[c] + i * g.xmat[c] + j * g.xmat[3 + c] + k * g.xmat[6 + c];
}

// one grd quantity per point from a (rho, grad, hess) record; the gradient
// is zero within 1e-5 bohr of a nucleus (src/fieldmod@proc.f90:1148-1154)
__global__ void k_field_prop(const double *__restrict__ rec, const double *__restrict__ xyz, long n, int prop,
                             const double4 *__restrict__ atoms, int natom, double *__restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double *r = rec + 10 * t;
  double g[3] = {r[1], r[2], r[3]};
  if (prop >= 1 && prop <= 4) {
    for (int a = 0; a < natom; a++) {
      const double4 A = atoms[a];
      const double dx = xyz[3 * t] - A.x, dy = xyz[3 * t + 1] - A.y, dz = xyz[3 * t + 2] - A.z;
      if (dx * dx + dy * dy + dz * dz <= 1e-10) g[0] = g[1] = g[2] = 0.0;
    }
  }
  double v;
  switch (prop) {
    case 0: v = r[0]; break;
    case 1: v = g[0]; break;
    case 2: v = g[1]; break;
    case 3: v = g[2]; break;
    case 4: v = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]); break;
    case 5: v = r[4]; break;  // hxx
    case 6: v = r[7]; break;  // hxy
    case 7: v = r[8]; break;  // hxz
    case 8: v = r[5]; break;  // hyy
    case 9: v = r[9]; break;  // hyz
    case 10: v = r[6]; break;  // hzz
    default: v = r[4] + r[5] + r[6]; break;  // laplacian
  }
  out[t] = v;
}

}  // namespace

void field_grid_dev(Handle &h, const GridSpec &g, int prec, int prop, double *d_out, cudaStream_t st) {
  const long plane = (long)g.nstep[1] * g.nstep[2];
  const int nip = (int)std::max(1L, std::min((long)g.nstep[0], (4L << 20) / std::max(1L, plane)));
  const long cap = (long)nip * plane;
  double *xyz = nullptr, *rec = nullptr;
  if (cudaMalloc(&xyz, sizeof(double) * 3 * cap) != cudaSuccess) fail(C2G_ERR_ALLOC, "cudaMalloc (grid points)");
  if (cudaMalloc(&rec, sizeof(double) * 10 * cap) != cudaSuccess) {
    cudaFree(xyz);
    fail(C2G_ERR_ALLOC, "cudaMalloc (grid records)");
  }
  try {
    for (int i0 = 0; i0 < g.nstep[0]; i0 += nip) {
      const int ni = std::min(nip, g.nstep[0] - i0);
      const long n = (long)ni * plane;
      k_grid_points<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, i0, n, xyz);
      C2G_CUDA(cudaGetLastError());
      if (prec == C2G_PREC_FP64) launch_fp64_points(h.dev, (int)n, xyz, 2, false, rec, st);
      else tc_points(h, prec, (int)n, xyz, rec, st);
      k_field_prop<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rec, xyz, n, prop, h.dev.atoms, h.dev.natom,
                                                                d_out + (long)i0 * plane);
      C2G_CUDA(cudaGetLastError());
    }
    C2G_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    cudaFree(xyz);
    cudaFree(rec);
    throw;
  }
  cudaFree(xyz);
  cudaFree(rec);
}

}  // namespace c2g
