/* Learned time-stepping surrogate for batched Acoustic2D parameter sweeps.
 *
 * A residual CNN of 3x3 convolutions jumps a 2-D staggered acoustic field (p, vx,
 * vy) K steps ahead; the finite-difference engine (fds_capi.h) generates its
 * training data, checks it periodically and takes over when it is off. The
 * reference (emtpb/pyfds) has no learned component: this library part serves the
 * parameter-sweep pattern built around Acoustic2D (pyfds/acoustics.py:89-128).
 *
 * Activations are bfloat16 in a channel-group blocked layout,
 * [batch][channels / 8][height][width][8] (the 8 channels of a group are one 16-byte
 * row per pixel), with channels a multiple of 16. Convolutions run on the fifth-generation tensor
 * cores (BF16 operands, FP32 accumulation in tensor memory); weights enter them
 * in a packed operand layout produced by fds_conv_pack / fds_adamw.
 *
 * All pointers are device pointers; every call is asynchronous on `stream` and
 * returns FDS_OK or an FDS_E_* code (fds_capi.h), with a message in fds_last_error.
 */
#ifndef FDS_SURROGATE_H
#define FDS_SURROGATE_H

#include <stddef.h>
#include <stdint.h>

#include "fds_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Convolution epilogues (FdsConvArgs.mode). */
#define FDS_CONV_FWD_GELU 0   /* z = conv(x) + bias -> out_z (optional); h = gelu(z) + resid -> out_h */
#define FDS_CONV_FWD_LINEAR 1 /* y = conv(x) + bias -> out_f32 (float32) */
#define FDS_CONV_BWD_DATA 2   /* g = conv(x, flipped transposed weights) + resid -> out_h (optional);
                                 dz = g * gelu'(zin) -> out_z */

/* Status bits OR-ed into *status by the kernels (a wait that gave up). */
#define FDS_SURR_STATUS_TIMEOUT 1
#define FDS_SURR_STATUS_ALIGN 2 /* shared memory not 128-byte aligned (nothing ran) */

typedef struct FdsConvArgs {
  int32_t batch, height, width; /* width a multiple of 128, height of 4 * dilation */
  int32_t cin, cout;            /* 16, 32 or 48 each */
  int32_t dilation;             /* 1, 2, 4 or 8 */
  int32_t mode;                 /* FDS_CONV_* */
  int32_t reserved;
  const void* x;      /* bf16 [B][cin/8][H][W][8] */
  const void* weight; /* bf16 packed operand, fds_conv_packed_elems(cin, cout) elements */
  const float* bias;  /* [cout] or NULL (forward modes) */
  const void* resid;  /* bf16 [B][cout/8][H][W][8] or NULL */
  const void* zin;    /* bf16 [B][cout/8][H][W][8]: pre-activation for gelu' (FDS_CONV_BWD_DATA) */
  void* out_z;        /* bf16 [B][cout/8][H][W][8] or NULL */
  void* out_h;        /* bf16 [B][cout/8][H][W][8] or NULL */
  float* out_f32;     /* float32 [B][cout/8][H][W][8] (FDS_CONV_FWD_LINEAR) */
  int32_t* status;    /* device int32 or NULL */
} FdsConvArgs;

/* Replaces nothing in the reference (see header comment). */
int32_t fds_conv3x3(const FdsConvArgs* args, void* stream);

/* Elements of a packed weight operand (9 * cin * cout). */
int64_t fds_conv_packed_elems(int32_t cin, int32_t cout);

/* Packs float32 master weights [9][cout][cin] (tap = 3*dy + dx) into the bf16
 * forward operand `wfwd` and, when non-NULL, the data-gradient operand `wbwd`
 * (the weights of the transposed convolution: taps flipped, cin and cout swapped). */
int32_t fds_conv_pack(int32_t cin, int32_t cout, const float* w, void* wfwd, void* wbwd,
                      void* stream);

typedef struct FdsWgradArgs {
  int32_t batch, height, width, cin, cout, dilation; /* as in FdsConvArgs; height a multiple of 2 * dilation */
  const void* x;     /* bf16 [B][cin/8][H][W][8]: the layer's input */
  const void* dz;    /* bf16 [B][cout/8][H][W][8]: gradient at the layer's pre-activation */
  float* partial;    /* [grid][9 * cout * cin + cout] float32: per-CTA weight and bias sums */
  int32_t grid;      /* CTAs (rows of `partial`); at most fds_conv_wgrad_max_grid() */
  int32_t reserved;
  int32_t* status;
} FdsWgradArgs;

/* Weight and bias gradient partial sums of one layer: partial[c] holds CTA c's
 * share of dW[tap][co][ci] = sum_p dz[p][co] x[p + offset(tap)][ci] and
 * db[co] = sum_p dz[p][co]. fds_adamw reduces the rows in a fixed order. */
int32_t fds_conv3x3_wgrad(const FdsWgradArgs* args, void* stream);
int32_t fds_conv_wgrad_max_grid(void);

typedef struct FdsAdamArgs {
  int32_t cin, cout;
  int32_t nparts; /* rows of `partial` */
  int32_t step;   /* 1-based optimiser step (bias correction) */
  float lr, beta1, beta2, eps, weight_decay;
  float grad_scale; /* multiplies the reduced gradient */
  const float* partial; /* [nparts][9 * cout * cin + cout] */
  float* weight;        /* float32 master [9][cout][cin] */
  float* bias;          /* float32 [cout] */
  float* m;             /* [9 * cout * cin + cout] first moments */
  float* v;             /* [9 * cout * cin + cout] second moments */
  void* wfwd;           /* bf16 packed forward operand (rewritten) */
  void* wbwd;           /* bf16 packed data-gradient operand (rewritten) or NULL */
  float* grad_out;      /* optional [9 * cout * cin + cout]: the reduced gradient */
} FdsAdamArgs;

/* Decoupled-weight-decay Adam step (Loshchilov & Hutter) on one layer, fused with
 * the reduction of the gradient partials and the repacking of the bf16 operands.
 * lr = 0 with grad_out set only reduces the gradient. */
int32_t fds_adamw(const FdsAdamArgs* args, void* stream);

/* ------------------------------------------------------------------ data plumbing */

typedef struct FdsSurrData {
  int32_t count;        /* samples in the batch */
  int32_t height, width;
  int32_t state_f64;    /* 1: state arrays are float64, 0: float32 */
  int32_t nsnap;        /* snapshots per instance in `state` */
  int32_t edge_zero_p;  /* unpack: pressure 0 on the outermost cells */
  const int32_t* inst;  /* [count] instance of each sample */
  const int32_t* snap;  /* [count] snapshot of each sample (target = snap + 1) */
  void* state;          /* [instances][nsnap][3][H][W] (p, vx, vy), flat x + y * W */
  const float* media;   /* [instances][2][H][W]: c dt/dx and rho / mean(rho) */
  const float* freq;    /* [instances] normalised source frequency */
  const float* zref;    /* [instances] impedance scale of the velocities */
  float* scale;         /* [count] energy norm of each input state */
  void* x;              /* bf16 [count][2][H][W][8] network input (16 channels) */
  float* s;             /* float32 [count][H][W][4] normalised input state */
  float* t;             /* float32 [count][H][W][4] normalised target, or NULL */
} FdsSurrData;

/* scale, then x / s (and t when set). */
int32_t fds_surr_pack(const FdsSurrData* d, void* stream);

/* pred = s + y[channels 0..2] (y float32 [count][2][H][W][8]); writes
 * dy = 2 (pred - t) / (count H W 3) as bf16 [count][2][H][W][8] (channels 3..15 zero) and per-CTA squared-error sums to
 * `loss_parts` (fds_surr_loss_parts(count, H, W) floats). */
int32_t fds_surr_loss(const FdsSurrData* d, const float* y, void* dy, float* loss_parts,
                      void* stream);
int32_t fds_surr_loss_parts(int32_t count, int32_t height, int32_t width);

/* state[inst][snap] = (s + y[channels 0..2]) de-normalised (the jump's result). */
int32_t fds_surr_unpack(const FdsSurrData* d, const float* y, void* stream);

/* Per sample: sums of squared differences and of squares of the energy-weighted
 * states a and b ([instances][3][H][W], float64, sample k at instance inst[k],
 * velocities times zref[inst[k]]);
 * out[2k] = |a - b|^2, out[2k + 1] = |b|^2. */
int32_t fds_surr_compare(int32_t count, int32_t height, int32_t width, const int32_t* inst,
                         const double* a, const double* b, const float* zref, double* out,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDS_SURROGATE_H */
