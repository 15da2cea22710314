/*
 * rift_closure.h -- C ABI of the learned sub-grid flux closure (no reference
 * counterpart: the reference solves on one grid and has no closure).
 *
 * A three-layer convolutional net reads six input channels around each cell
 * of a 2x-coarsened grid and predicts corrections to four face fluxes of
 * that cell:
 *   inputs  (h, hu, hv, b, n, rain), channel 3 entering as the bed elevation
 *           of each stencil cell minus that of the output cell;
 *   layer 1 6 -> 32 channels, 5x5, ReLU;
 *   layer 2 32 -> 32 channels, 3x3, ReLU;
 *   layer 3 32 -> 4 channels, 1x1;
 *   outputs (east-face mass flux, east-face x-momentum flux, north-face mass
 *           flux, north-face y-momentum flux), per unit face width.
 * Layers 1 and 2 run on the BF16 tensor cores with FP32 accumulation
 * (tcgen05.mma with tensor-memory accumulators in the forward and apply
 * kernels; the training kernel's forward and backward passes on mma.sync);
 * layer 3 of the forward and apply kernels runs in FP32.  The parameters are
 * one FP32 vector (RIFT_CLOSURE_NPARAM floats) laid out as below, rounded to
 * BF16 when a kernel stages them for a tensor-core layer.
 *
 * Every pointer argument is a device pointer unless it says host; `stream`
 * is a cudaStream_t (NULL: the legacy default stream).  Calls are
 * asynchronous on `stream` and return RIFT_OK or a RIFT_ERR_* code of
 * rift_gb300.h; rift_closure_last_error() gives the message of the calling
 * thread's last failure.
 */
#ifndef RIFT_CLOSURE_H
#define RIFT_CLOSURE_H

#include <stddef.h>
#include <stdint.h>
#include "rift_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- parameter vector (FP32) ------------------------------------------ */
/* W1[o][k], o < 32, k = (dy*5 + dx)*6 + c for k < 150, columns 150..159 zero */
#define RIFT_CLOSURE_OFF_W1 0
#define RIFT_CLOSURE_OFF_B1 5120
/* W2[o][k], k = (dy*3 + dx)*32 + c */
#define RIFT_CLOSURE_OFF_W2 5152
#define RIFT_CLOSURE_OFF_B2 14368
/* W3[o][c], rows 4..7 unused (zero) */
#define RIFT_CLOSURE_OFF_W3 14400
#define RIFT_CLOSURE_OFF_B3 14656
#define RIFT_CLOSURE_NPARAM 14664

/* Input channels: planes of FP32 values, sample s, row y, column x at
 * plane[c][s*sample_stride + y*pitch + x]; a NULL plane reads value[c]
 * everywhere.  Each value is multiplied by scale[c] before the net sees it.
 * Reads outside rows [0, H) or columns [0, W) are clamped to the edge.
 * Outputs are computed for the cells oy0 <= y < oy0+OH, ox0 <= x < ox0+OW of
 * each of `samples` samples. */
typedef struct rift_closure_src {
    const float* plane[6];
    float value[6];
    float scale[6];
    int64_t sample_stride;
    int32_t pitch;
    int32_t H, W;
    int32_t oy0, ox0, OH, OW;
    int32_t samples;
} rift_closure_src;

/* Net outputs, unscaled: out[((s*4 + ch)*OH + y)*OW + x] for output cell
 * (oy0 + y, ox0 + x) of sample s. */
int rift_closure_forward(const rift_closure_src* src, const float* params, float* out,
                         void* stream);

/* One pass of the loss and its gradient over every output cell of `src`:
 * loss = loss_scale * sum w * (out - target)^2 over samples, channels and
 * cells, target and w laid out like rift_closure_forward's output.
 * Adds d loss / d params to grad (NPARAM floats) and the loss to *loss
 * (one device double).  The caller zeroes both before the first pass of an
 * optimiser step. */
int rift_closure_train(const rift_closure_src* src, const float* params, const float* target,
                       const float* weight, float loss_scale, float* grad, double* loss,
                       void* stream);

/* Adam on n parameters; bias1 = 1 - beta1^step, bias2 = 1 - beta2^step.
 * Zeroes grad after reading it. */
int rift_closure_adam(float* params, float* grad, float* m, float* v, int32_t n, float lr,
                      float beta1, float beta2, float eps, float bias1, float bias2,
                      void* stream);

/* Adds weight x (central-upwind flux through the east and north face of
 * every interior cell) of a handle's current state (U^n of `view`) to acc,
 * four planes of acc_rows x acc_pitch floats: east mass, east x-momentum,
 * north mass, north y-momentum, per unit face width.  ratio 1: acc is on
 * the view's own grid.  ratio 2: acc is on the grid coarsened 2x (interior
 * cell (J, I) covers fine interior cells 2(J-2)+2.. and 2(I-2)+2..); each
 * coarse face gets the mean of the two fine faces on it.  The coarse grid
 * has acc_nx x acc_ny h-grid cells (ghost ring included). */
int rift_closure_face_flux(const rift_device_view* view, int32_t ratio, float weight, float* acc,
                           int32_t acc_pitch, int32_t acc_rows, int32_t acc_nx, int32_t acc_ny);

/* The closure step on a handle's grid: evaluates the net on every 16 x 16
 * block of interior cells that holds a cell deeper than hmin, turns its
 * outputs (times oscale[ch]) into face corrections and applies them to U^n
 * as antisymmetric fluxes over dtw seconds:
 *   h_p  -= dtw/dx (cE_p - cE_west) + dtw/dy (cN_p - cN_south), and the
 *   x (y) momentum likewise with the east (north) momentum correction.
 * A face is corrected only when both its cells are deeper than hmin and lie
 * at least one cell inside the ghost ring; its mass correction is limited
 * to lim x (donor depth) x dx / dtw.  A block whose largest ratio
 * |c_mass| dtw / (dx h_donor) exceeds tau falls back to the plain solve
 * (no correction).  src: the six input channels on the handle's grid
 * (plane[0..2] = the view's h, hu, hv); corr: four planes of the view's
 * layout (scratch, left holding the corrections computed per block);
 * block_fell: one byte per 16 x 16 block of interior cells, row-major over
 * ceil((h_nx-4)/16) blocks per row (scratch, left holding 1 for the blocks
 * that fell back).  A face between a block that fell back and one that did
 * not is not corrected either, so every cell of a block that fell back keeps
 * the plain solve exactly.  counters[0] += blocks evaluated, counters[1] +=
 * blocks fallen back.  lim < 0.25 and hmin (1 - 4 lim) > 1.19e-7 m, so that
 * no wet cell is dried (RIFT_ERR_ARG otherwise).  Runs on the view's
 * stream. */
int rift_closure_apply(const rift_device_view* view, const rift_closure_src* src,
                       const float* params, const float* oscale_host, float dtw, float hmin,
                       float lim, float tau, float* corr, uint8_t* block_fell, int32_t* counters);

/* Waits for `stream`, then reports (and clears) the device status of the
 * tensor-core kernels: RIFT_ERR_CUDA when a completion wait of one of them
 * gave up (its tile's outputs are then missing), else RIFT_OK.  The status
 * is one flag per device for the whole process, so a check after one
 * stream's launches also reports a give-up in kernels of another stream.
 * While the flag is set, rift_closure_apply changes no state (the step keeps
 * the plain solve). */
int rift_closure_check(void* stream);

/* One tensor-core MMA (128 x 32 x 16, BF16 in, FP32 out) on fixed values in
 * the forward pass's operand layout; out (device, 128 x 32 FP32, row-major)
 * receives the product A B^T with A[r][k] = (r % 7) - 3 + (k % 5) / 4 and
 * B[n][k] = (n % 5) - 2 + (k % 3) / 2, exact in FP32.  For start-up checks. */
int rift_closure_selftest(float* out, void* stream);

const char* rift_closure_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* RIFT_CLOSURE_H */
