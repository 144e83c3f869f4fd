/*
 * critic2_gb300 -- C ABI of the learned critical-point seed proposer.
 *
 * These entries have no counterpart in the reference: critic2's AUTO seeds
 * its Newton searches geometrically (pair seeds, src/autocp@proc.f90:
 * 423-437).  Here a small 3D convolutional network proposes seeds from a
 * coarse grid of the density; its seeds then go through the unchanged
 * Newton + addcp stages (c2g_autocritic with explicit seeds), and the
 * caller keeps plain pair seeding as the fallback when the resulting CP
 * list fails the Poincare-Hopf check.
 *
 * All pointers are device pointers (allocated by the caller) unless stated;
 * `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 * asynchronous on the stream.  Tensors are channel-last FP32,
 * x[b][d][h][w][c]; convolutions are "same" (zero padding), stride 1, with
 * weights w[tap][cin][cout], tap = (kz*k + ky)*k + kx (kz along d).
 * Every entry returns a C2G_* status (include/critic2_gb300.h).
 */
#ifndef CRITIC2_GB300_CPSEED_H
#define CRITIC2_GB300_CPSEED_H

#ifdef __cplusplus
extern "C" {
#endif

/* y[b][v][cout] = bias + sum over taps and cin of x * w, optional ReLU.
 * cin in {4, 8, 16, 32}, cout in {8, 16, 32}, ksize 1 or 3, W even. */
int c2g_cs_conv3d(const float *x, int B, int D, int H, int W, int cin, const float *w, const float *bias,
                  int cout, int ksize, int relu, float *y, void *stream);

/* Input gradient of c2g_cs_conv3d: dx = conv(dy, flipped, transposed w),
 * multiplied by (mask > 0) when mask (shape of dx) is not NULL -- the ReLU
 * derivative of the layer that produced x.  cin a multiple of 8. */
int c2g_cs_conv3d_bwd_data(const float *dy, int B, int D, int H, int W, int cout, const float *w, int cin,
                           int ksize, const float *mask, float *dx, void *stream);

/* Weight and bias gradients of c2g_cs_conv3d, ADDED to dw[tap][cin][cout]
 * and db[cout] (db may be NULL). */
int c2g_cs_conv3d_bwd_weight(const float *x, const float *dy, int B, int D, int H, int W, int cin, int cout,
                             int ksize, float *dw, float *db, void *stream);

/* Loss of the proposer's 8-channel output per voxel (channels 0-3 CP-type
 * heat-map logits: non-nuclear maximum, bond, ring, cage; 4-6 sub-voxel
 * offsets; 7 unused) against targets of the same shape (0-3 labels, 4-6
 * offsets, 7 = 1 on labelled voxels): weighted binary cross-entropy (mean
 * over voxels, positives weighted by pos_weight) + off_weight * squared
 * offset error / 2 averaged over npos labelled voxels.  Writes dlogits and
 * ADDS the loss to *d_loss. */
int c2g_cs_loss(const float *logits, const float *tgt, long nvox, int npos, float pos_weight,
                float off_weight, float *dlogits, double *d_loss, void *stream);

/* Dense targets from cps[n][5] = (sample, fi, fj, fk, type) in fractional
 * voxel coordinates of an S^3 grid per sample: the 8 voxels around each CP
 * get label `type` (0-3) and their offset to the CP.  tgt[B][S^3][8] must
 * be zero on entry. */
int c2g_cs_targets(const float *d_cps, int ncp, int S, float *tgt, void *stream);

/* Network input from an NCI grid (d_crho = sign(lambda2) rho * 100, d_cgrad
 * = s, as written by c2g_nciplot_dev): x[v][4] = ((clamp(log10 rho, -12,
 * 4) + 4) / 4, sign(lambda2), -clamp(log10 s, -4, 2) / 2, 0). */
int c2g_cs_features(const double *d_crho, const double *d_cgrad, long nvox, float *x, void *stream);

/* Seeds from the network's output on one S^3 grid whose voxel (i,j,k) is
 * at x0 + h*(i,j,k) (x0 a HOST array of 3).  mode 0: every voxel whose
 * largest heat-map logit exceeds thresh_logit; 1: ... that is also a
 * maximum of the largest logit over its 26 neighbours; 2: voxels where some
 * CP type's logit exceeds thresh_logit and is a maximum of that type's map
 * over the 26 neighbours; 3: as 2 over the 6 face neighbours.  A seed is
 * the voxel plus the predicted offset.  Writes up to cap seeds d_seeds(3,*)
 * and their voxel indices, *d_count = number found (may exceed cap). */
int c2g_cs_seeds(const float *logits, int S, const double *x0, double h, float thresh_logit, int mode,
                 int cap, double *d_seeds, int *d_vox, int *d_count, void *stream);

/* One Adam step (bias-corrected, step t >= 1) on n parameters. */
int c2g_cs_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                int t, void *stream);

#ifdef __cplusplus
}
#endif

#endif
