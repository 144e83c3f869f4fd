// critic2's NCI checkpoint file (<root>.chk_nci): writechk / readchk,
// src/nci@proc.f90:1019-1117.  The file is Fortran unformatted sequential
// (gfortran layout, 4-byte record markers, little-endian on both hosts):
//   (llat, llfrag, nfrag)  3 x int32, logicals as 0/1
//   x0(3), xmat(:,1), xmat(:,2), xmat(:,3)   4 records of 3 doubles
//   nstep(3)               3 x int32
//   crho, cgrad            one record, 2 n doubles, (k,j,i) order
//   [rhoat], [rhofrag]     only when the promolecular arrays exist
// A record longer than 2^31 - 9 bytes is split into subrecords: the leading
// marker of every subrecord but the last is negative, the trailing marker
// of every subrecord but the first is negative (libgfortran's convention;
// the reader accepts either sign on either marker).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "c2g_internal.h"

namespace c2g {
namespace {

constexpr int64_t kMaxSubrecord = 2147483639;  // 2 GiB - 9

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

void put_marker(FILE *f, int32_t m, const std::string &path) {
  if (std::fwrite(&m, 4, 1, f) != 1) fail(C2G_ERR_IO, "write failed: " + path);
}

// One record made of the concatenation of the given byte ranges.
void write_record(FILE *f, const std::vector<std::pair<const void *, size_t>> &parts, const std::string &path) {
  size_t total = 0;
  for (auto &p : parts) total += p.second;
  size_t part = 0, off = 0, done = 0;
  bool first = true;
  do {
    const size_t len = (size_t)std::min<int64_t>((int64_t)(total - done), kMaxSubrecord);
    const bool last = done + len == total;
    put_marker(f, last ? (int32_t)len : -(int32_t)len, path);
    size_t left = len;
    while (left > 0) {
      const size_t n = std::min(left, parts[part].second - off);
      if (n && std::fwrite(static_cast<const char *>(parts[part].first) + off, 1, n, f) != n)
        fail(C2G_ERR_IO, "write failed: " + path);
      off += n;
      left -= n;
      if (off == parts[part].second) part++, off = 0;
    }
    put_marker(f, first ? (int32_t)len : -(int32_t)len, path);
    done += len;
    first = false;
  } while (done < total);
}

// Reads one record (all its subrecords) into the destination ranges, in
// order; bytes beyond them are skipped, as a Fortran READ of fewer items
// than the record holds.  Returns the record's length, or -1 at end of file.
int64_t read_record(FILE *f, const std::vector<std::pair<void *, size_t>> &dst, const std::string &path) {
  size_t part = 0, off = 0;
  int64_t total = 0;
  bool more = true;
  while (more) {
    int32_t lead = 0, trail = 0;
    if (std::fread(&lead, 4, 1, f) != 1) {
      if (total == 0 && part == 0 && off == 0) return -1;
      fail(C2G_ERR_IO, "truncated record in " + path);
    }
    int64_t left = lead < 0 ? -(int64_t)lead : (int64_t)lead;
    const int64_t len = left;
    char skip[4096];
    while (left > 0) {
      size_t n;
      char *to;
      if (part < dst.size()) {
        n = (size_t)std::min<int64_t>(left, (int64_t)(dst[part].second - off));
        to = static_cast<char *>(dst[part].first) + off;
      } else {
        n = (size_t)std::min<int64_t>(left, (int64_t)sizeof(skip));
        to = skip;
      }
      if (n && std::fread(to, 1, n, f) != n) fail(C2G_ERR_IO, "truncated record in " + path);
      left -= (int64_t)n;
      if (part < dst.size()) {
        off += n;
        if (off == dst[part].second) part++, off = 0;
      }
    }
    if (std::fread(&trail, 4, 1, f) != 1) fail(C2G_ERR_IO, "truncated record in " + path);
    if ((trail < 0 ? -(int64_t)trail : (int64_t)trail) != len) fail(C2G_ERR_IO, "bad record marker in " + path);
    total += len;
    more = lead < 0;
  }
  return total;
}

}  // namespace
}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_nci_chk_write(const char *path, const double *x0, const double *xmat, const int *nstep,
                      const double *crho, const double *cgrad) {
  return guarded([&] {
    if (!path || !x0 || !xmat || !nstep || !crho || !cgrad) fail(C2G_ERR_ARG, "null argument");
    for (int j = 0; j < 3; j++)
      if (nstep[j] <= 0) fail(C2G_ERR_ARG, "nstep must be positive");
    const size_t n = (size_t)nstep[0] * nstep[1] * nstep[2];
    const std::string p(path);
    File fh;
    fh.f = std::fopen(path, "wb");
    if (!fh.f) fail(C2G_ERR_IO, "cannot open " + p);
    const int32_t head[3] = {0, 0, 0};  // no promolecular or fragment arrays
    write_record(fh.f, {{head, sizeof(head)}}, p);
    write_record(fh.f, {{x0, 3 * sizeof(double)}}, p);
    for (int j = 0; j < 3; j++) write_record(fh.f, {{xmat + 3 * j, 3 * sizeof(double)}}, p);
    const int32_t ns[3] = {nstep[0], nstep[1], nstep[2]};
    write_record(fh.f, {{ns, sizeof(ns)}}, p);
    write_record(fh.f, {{crho, n * sizeof(double)}, {cgrad, n * sizeof(double)}}, p);
    if (std::fclose(fh.f) != 0) {
      fh.f = nullptr;
      fail(C2G_ERR_IO, "write failed: " + p);
    }
    fh.f = nullptr;
  });
}

int c2g_nci_chk_read(const char *path, const double *x0, const double *xmat, const int *nstep, double *crho,
                     double *cgrad, int *found) {
  return guarded([&] {
    if (!path || !x0 || !xmat || !nstep || !crho || !cgrad || !found) fail(C2G_ERR_ARG, "null argument");
    *found = 0;
    const std::string p(path);
    File fh;
    fh.f = std::fopen(path, "rb");
    if (!fh.f) return;  // no checkpoint: not an error (readchk's lchk = .false.)
    auto need = [&](const std::vector<std::pair<void *, size_t>> &dst) {
      size_t bytes = 0;
      for (auto &d : dst) bytes += d.second;
      const int64_t len = read_record(fh.f, dst, p);
      if (len < (int64_t)bytes) fail(C2G_ERR_IO, "truncated checkpoint " + p);
    };
    int32_t head[3];
    need({{head, sizeof(head)}});
    // the caller has no promolecular or fragment arrays (nfrag = 0)
    if (head[2] != 0) return;
    double v[3];
    need({{v, sizeof(v)}});
    for (int j = 0; j < 3; j++)
      if (std::fabs(v[j] - x0[j]) > 1e-13) return;
    for (int c = 0; c < 3; c++) {
      need({{v, sizeof(v)}});
      for (int j = 0; j < 3; j++)
        if (std::fabs(v[j] - xmat[3 * c + j]) > 1e-13) return;
    }
    int32_t ns[3];
    need({{ns, sizeof(ns)}});
    for (int j = 0; j < 3; j++)
      if (ns[j] != nstep[j]) return;
    const size_t n = (size_t)nstep[0] * nstep[1] * nstep[2];
    need({{crho, n * sizeof(double)}, {cgrad, n * sizeof(double)}});
    *found = 1;
  });
}

}  // extern "C"
