// Split-precision evaluator (placeholder until the tcgen05 kernel lands).
#include "k_tc.h"

namespace c2g {

struct TcOperands {
  int dummy;
};

TcOperands *tc_create(Handle &) { return new TcOperands{0}; }
void tc_destroy(TcOperands *t) { delete t; }

void tc_points(Handle &, int, int, const double *, double *, cudaStream_t) {
  fail(C2G_ERR_UNSUPPORTED, "split-precision evaluation is not built yet");
}

void tc_points_index(Handle &, int, const double *, const int *, const int *, int, double *,
                     cudaStream_t) {
  fail(C2G_ERR_UNSUPPORTED, "split-precision evaluation is not built yet");
}

long tc_nci_grid(Handle &, int, const GridSpec &, double *, double *, cudaStream_t, cudaEvent_t) {
  fail(C2G_ERR_UNSUPPORTED, "split-precision evaluation is not built yet");
}

}  // namespace c2g
