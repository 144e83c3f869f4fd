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

void fix_flags(const int *d_flags, const int *d_nflag, const double *d_v, char *text, bool on_device, bool cube,
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
    char buf[16];
    long off;
    int len;
    if (cube) {
      const long rec = i / n3;
      const int m = (int)(i - rec * n3);
      off = rec * rec_bytes + 14L * m + m / 6;
      fmt_e13_5e3(x, buf);
      len = 14;
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
    fix_flags(flags, nflag, d_v, h_text, false, true, nstep[2], rb, st);
  } else {
    fix_flags(flags, nflag, d_v, d_text, true, true, nstep[2], rb, st);
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
    fix_flags(flags, nflag, d_dat, h_text, false, false, 0, 0, st);
  } else {
    fix_flags(flags, nflag, d_dat, d_text, true, false, 0, 0, st);
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

}  // namespace c2g
