/*
 * swlearn.h — learned 2x frame upscaler of the GB300 renderer (part of libswgpu.so).
 *
 * No counterpart in the reference: the reference's FrameUpscaler (src/square_wheel/frame_upscaler.rs)
 * only has nearest and 2x-averaging upscales (sw_upscale modes SW_UPSCALE_NEAREST / SW_UPSCALE_AVG2X);
 * this is the learned form that replaces them. A frame is rendered at half resolution, tonemapped to
 * Color32, and a small convolutional network restores full resolution:
 *
 *   x = (b, g, r) / 255 of the half-resolution frame (3 channels)
 *   conv3x3 3->32 + ReLU, conv3x3 32->32 + ReLU, conv3x3 32->32 + ReLU, conv3x3 32->12
 *   (zero padding), pixel shuffle 2x (channel c*4 + sy*2 + sx -> colour c of output pixel
 *   (2x+sx, 2y+sy)), plus a bilinear 2x upsample of x (weights 3/4, 1/4, edges clamped)
 *   output byte = clamp(round(255 * value), 0, 255); alpha copied from the source pixel.
 *
 * BF16 weights and activations with FP32 accumulation on the tensor cores (tcgen05.mma); training
 * (forward, backward, Adam) runs in the library's own kernels. Parameters are exchanged in a canonical
 * FP32 layout: for each layer l = 0..3, weights [c_out][ky][kx][c_in] then bias [c_out]
 * (SW_UPSCALER_NUM_PARAMS values in total).
 *
 * Every function returns 0 or a negative SwStatus and never aborts.
 */
#ifndef SWLEARN_H
#define SWLEARN_H

#include "swgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SW_UPSCALER_NUM_PARAMS 22860u
#define SW_UPSCALER_CROP_W 128u   /* training crop, half-resolution pixels */
#define SW_UPSCALER_CROP_H 64u
#define SW_UPSCALER_CROP_MARGIN 4u /* crop border pixels left out of the loss (receptive-field radius) */
#define SW_UPSCALER_MAX_CROPS 32u

typedef struct SwUpscaler SwUpscaler;

/* One training crop: a SW_UPSCALER_CROP_W x SW_UPSCALER_CROP_H window at (x, y) of a half-resolution
 * frame `lo` and the matching full-resolution frame `hi` (2*lo_width x 2*lo_height). Device pointers to
 * Color32 pixels; pitches in pixels. The window must lie inside the frame. */
typedef struct SwUpscalerCrop {
	const uint32_t* lo;
	const uint32_t* hi;
	uint32_t lo_width, lo_height, lo_pitch, hi_pitch;
	int32_t x, y;
} SwUpscalerCrop;

/* New network on `device` with seeded He-normal weights (zero biases, last layer scaled by 1/10),
 * Adam state zeroed. Inference buffers are sized on first use. */
int sw_upscaler_create(int device, uint64_t seed, SwUpscaler** out);
int sw_upscaler_destroy(SwUpscaler* ups);
const char* sw_upscaler_last_error(const SwUpscaler* ups);

/* Canonical FP32 parameters (count must be SW_UPSCALER_NUM_PARAMS). set_params resets Adam. */
int sw_upscaler_get_params(SwUpscaler* ups, float* params, uint32_t count);
int sw_upscaler_set_params(SwUpscaler* ups, const float* params, uint32_t count);

/* Forward + backward over the crops without an update: gradients of
 *   loss = 0.5 * sum(diff^2) / n,  diff = network output - hi frame value (both in [0, 1] units),
 * n = the number of (pixel, colour) pairs inside the crops' loss windows, in the canonical layout.
 * grads (host, SW_UPSCALER_NUM_PARAMS floats) and loss (host, may be NULL) are written on return. */
int sw_upscaler_gradients(SwUpscaler* ups, const SwUpscalerCrop* crops, uint32_t num_crops, float* grads, float* loss);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at learning rate lr on the crops' loss. If mse is
 * not NULL the call waits for the step and writes mean(diff^2); otherwise it is asynchronous. */
int sw_upscaler_train_step(SwUpscaler* ups, const SwUpscalerCrop* crops, uint32_t num_crops, float lr, float* mse);
/* Adam steps taken so far. */
int sw_upscaler_steps(SwUpscaler* ups, uint64_t* out_steps);

/* Upscale a half-resolution Color32 frame lo (device, lo_width x lo_height, lo_pitch pixels per row) into
 * hi (device, 2*lo_width x 2*lo_height, hi_pitch). stream: cudaStream_t, NULL = the upscaler's own
 * stream. Asynchronous. */
int sw_upscaler_infer(SwUpscaler* ups, const uint32_t* lo, uint32_t lo_width, uint32_t lo_height, uint32_t lo_pitch,
	uint32_t* hi, uint32_t hi_pitch, void* stream);

/* Inference by one fused kernel for all four layers (1, default; activations stay in shared memory) or
 * by one launch per layer (0; activations through HBM). Both give the same bytes. */
int sw_upscaler_set_fused(SwUpscaler* ups, int enable);
/* Wait for the device and report whether any upscaler kernel gave up on a bounded wait. */
int sw_upscaler_check(SwUpscaler* ups);
/* Failure-detection check of the bounded waits (no counterpart in the reference): one kernel arms an
 * mbarrier that nothing completes (no copy or MMA in flight), waits at most max_polls polls
 * (1..2^21), and takes the upscaler kernels' recovery path - error code 5 recorded, TMEM freed, return.
 * *out_code receives the recorded code (5 when the wait ran out); the record is then cleared, so the
 * upscaler stays usable. Fails with SW_ERR_STATE if an earlier kernel's failure is still recorded. */
int sw_upscaler_wait_probe(SwUpscaler* ups, uint32_t max_polls, int* out_code);

/* PSNR (dB, colour channels b, g, r) between two device Color32 frames; 99 when identical. Waits. */
int sw_upscaler_psnr(SwUpscaler* ups, const uint32_t* a, uint32_t a_pitch, const uint32_t* b, uint32_t b_pitch,
	uint32_t width, uint32_t height, void* stream, double* out_psnr);

/* Checkpoint: parameters, Adam moments and step count in a versioned binary file with an FNV-1a 64
 * hash of the payload; load rejects a file whose version, size or hash does not match. */
int sw_upscaler_save(SwUpscaler* ups, const char* path);
int sw_upscaler_load(SwUpscaler* ups, const char* path);

/* Use `ups` for sw_upscale(ctx, SW_UPSCALE_LEARNED, 2, ...) on the context's stream (NULL detaches). */
int sw_set_learned_upscaler(SwCtx* ctx, SwUpscaler* ups);

/* Every-Nth-frame quality monitor of the learned path (host logic, no GPU). Per frame the caller asks
 * sw_monitor_plan what to render:
 *   SW_PLAN_LEARNED           half resolution + learned upscale
 *   SW_PLAN_LEARNED_CHECKED   the same plus a plain full-resolution frame; report the PSNR between them
 *                             with sw_monitor_report
 *   SW_PLAN_PLAIN             plain full resolution (fallback)
 * A check below threshold_db switches to the plain path for fallback_frames frames; the first frame
 * after that is checked again. */
typedef struct SwMonitor {
	uint32_t check_interval;  /* N: every Nth learned frame is checked (>= 1) */
	uint32_t fallback_frames; /* plain frames after a failed check (>= 1) */
	float threshold_db;
	/* state */
	uint64_t frames, learned_frames, checks, failed_checks, fallbacks, plain_frames;
	uint32_t plain_left;    /* plain frames still to render */
	uint32_t since_check;   /* learned frames since the last check */
	uint32_t check_pending; /* a checked frame awaits its report */
	uint32_t recheck;       /* check the next learned frame */
	float last_psnr_db;
} SwMonitor;

enum SwMonitorPlan {
	SW_PLAN_LEARNED = 0,
	SW_PLAN_LEARNED_CHECKED = 1,
	SW_PLAN_PLAIN = 2,
};

int sw_monitor_init(SwMonitor* m, uint32_t check_interval, float threshold_db, uint32_t fallback_frames);
int sw_monitor_plan(SwMonitor* m, uint32_t* out_plan);
int sw_monitor_report(SwMonitor* m, double psnr_db);

#ifdef __cplusplus
}
#endif

#endif /* SWLEARN_H */
