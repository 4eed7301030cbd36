/* usx_cu.h — C-ABI of the GB300 (sm_103a) imaging path.
 *
 * This is the boundary the host layer (the C++ classes behind the `_usx`
 * module, or any FFI: ctypes, cgo, JNI) calls. It takes plain pointers, sizes
 * and the POD descriptors of usx_types.h; no C++ or torch types cross it.
 *
 * Conventions
 *  - Every entry point returns USX_OK (0) or a USX_ERR_* code; the message of
 *    the last failure on the calling thread is usx_cu_last_error(). Invalid
 *    arguments map to USX_ERR_INVALID, the way the reference throws
 *    std::invalid_argument (types.cpp:8-124, beamformer.cpp:218-225).
 *  - Sample and image buffers are DEVICE pointers on the context's device;
 *    descriptors (transmits, grid axes) are HOST memory read during the call.
 *  - Work is enqueued on the context's stream; calls return without waiting
 *    unless they must read a device result back (documented per function).
 *  - Complex data is interleaved float (re, im), i.e. std::complex<float>.
 *  - Layouts follow the reference: channel data [event][channel][sample],
 *    frames [axis0][axis1] with axis1 fastest, grid points [pixel][x,y,z].
 */
#ifndef USX_CU_H
#define USX_CU_H

#include "usx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  USX_OK = 0,
  USX_ERR_INVALID = 1,      /* bad argument (reference: std::invalid_argument) */
  USX_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  USX_ERR_NOMEM = 3,        /* device allocation failed */
  USX_ERR_NUMERIC = 4,      /* a kernel reported a numeric failure */
  USX_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  USX_ERR_UNSUPPORTED = 6   /* configuration outside what the kernels implement */
};

#define USX_CU_ABI_VERSION 1

typedef struct usx_ctx usx_ctx;
typedef struct usx_bf_plan usx_bf_plan;
typedef struct usx_mlp usx_mlp;

/* ----------------------------------------------------------- context, memory */

int usx_cu_abi_version(void);
/* Compute capability of the device code the library loaded on the current
 * device, major * 10 + minor (103 for sm_103a). Needs a device. */
int usx_cu_binary_version(int* version);
/* Message of the last failed call on this thread ("" if none). */
const char* usx_cu_last_error(void);

/* One context per device and host thread of use. The context owns a stream
 * (or adopts `stream` if non-NULL; a cudaStream_t) and a grow-only scratch
 * arena. */
int usx_cu_ctx_create(int device, void* stream, usx_ctx** out);
int usx_cu_ctx_destroy(usx_ctx* ctx);
void* usx_cu_ctx_stream(usx_ctx* ctx);
int usx_cu_ctx_set_stream(usx_ctx* ctx, void* stream);
int usx_cu_synchronize(usx_ctx* ctx);

int usx_cu_malloc(usx_ctx* ctx, size_t bytes, void** dev);
int usx_cu_free(usx_ctx* ctx, void* dev);
/* Page-locked host memory, for host buffers that are copied every frame. */
int usx_cu_host_alloc(usx_ctx* ctx, size_t bytes, void** host);
int usx_cu_host_free(usx_ctx* ctx, void* host);
/* Copies on the context's stream; *_sync variants wait for completion. */
int usx_cu_memcpy_h2d(usx_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes);
int usx_cu_memcpy_d2h(usx_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes);
int usx_cu_memcpy_d2d(usx_ctx* ctx, void* dst_dev, const void* src_dev, size_t bytes);
int usx_cu_memset(usx_ctx* ctx, void* dst_dev, int value, size_t bytes);

/* Per-kernel timing with CUDA events recorded on the context's stream around
 * every launch (off by default; no counterpart in the reference, whose only
 * timing is PipelineStats' wall clock, pipeline.cpp:25-46). profile_read
 * returns the index-th distinct kernel name with its summed device time and
 * launch count, and USX_ERR_INVALID past the last one. */
int usx_cu_profile_enable(usx_ctx* ctx, int on);
int usx_cu_profile_reset(usx_ctx* ctx);
int usx_cu_profile_read(usx_ctx* ctx, int index, char* name, int name_cap, double* total_ms,
                        int64_t* launches);

/* ------------------------------------------------------------------ simulator */

/* Simulator::simulate (reference simulator.cpp:213-419): point scatterers ->
 * RF [n_events][n_elements][n_samples] float, overwritten. `scat` is a device
 * array of n_scat usx_scatterer. `noise_z` is NULL (no receive noise) or a
 * device array of n_events*n_elements*n_samples standard normals, the draws of
 * std::normal_distribution<float> seeded noise_seed+event (simulator.cpp:
 * 406-415); each event adds z * peak * 10^(noise_db/20). `stats` (host, may be
 * NULL) receives {scatterer-element-samples accumulated, flops} of the call
 * and forces a synchronisation when given. */
int usx_cu_simulate(usx_ctx* ctx, const usx_channel_desc* cd, const usx_simulator_config* cfg,
                    const usx_scatterer* scat, int64_t n_scat, const float* noise_z, float* rf,
                    double* stats);

/* Simulator::pulse (simulator.cpp:140-154), computed on the host: writes up to
 * `cap` taps to `out` (host) and returns the tap count via *n_taps. */
int usx_cu_pulse(const usx_probe* probe, const usx_acquisition* acq,
                 const usx_simulator_config* cfg, float* out, int cap, int* n_taps,
                 float* half_duration);

/* ---------------------------------------------------------------- demodulator */

/* demodulate (reference demodulate.cpp:36-121): RF [E][C][N] float ->
 * IQ [E][C][ceil(N/dec)] complex. *out_fdem receives the demodulation
 * frequency used (config value, else the probe centre frequency). */
int usx_cu_demodulate(usx_ctx* ctx, const usx_channel_desc* cd, const usx_demod_config* cfg,
                      const float* rf, float* iq, float* out_fdem);

/* design_lowpass (demodulate.cpp:13-34), host-side; returns taps via *n_taps. */
int usx_cu_design_lowpass(int n_taps, float normalized_cutoff, float* h, int cap, int* n_out);

/* ----------------------------------------------------------------- beamformer */

/* A beamforming plan: the channel metadata, grid and config of
 * Beamformer::beamform (reference beamformer.cpp:297-549) frozen on the device
 * (transmit tables, pixel positions), so that executing it only launches
 * kernels and can be captured in a CUDA graph. `points_host` is the grid's
 * point list [n_axis0*n_axis1][3] (host memory, copied). */
int usx_cu_bf_plan_create(usx_ctx* ctx, const usx_channel_desc* cd, const usx_grid_desc* grid,
                          const float* points_host, const usx_beamformer_config* cfg,
                          int event_begin, int event_end, usx_bf_plan** out);
int usx_cu_bf_plan_destroy(usx_bf_plan* plan);
/* Device bytes of scratch one execution of the plan needs (MV snapshots). */
int usx_cu_bf_plan_workspace(const usx_bf_plan* plan, size_t* bytes);
/* Beamform one acquisition: `data` is RF float or IQ complex as the plan's
 * channel descriptor says; `frame` receives n_axis0*n_axis1 complex. */
int usx_cu_bf_execute(usx_bf_plan* plan, const void* data, float* frame);
/* Beamform `n_frames` acquisitions laid out back to back (strides in
 * elements of the data type: floats for RF, complex for IQ; frames in complex)
 * in one launch sequence. */
int usx_cu_bf_execute_batch(usx_bf_plan* plan, int n_frames, const void* data,
                            int64_t data_stride, float* frames, int64_t frame_stride);

/* Arithmetic of the delay-and-sum stage (no counterpart in the reference):
 *   USX_BF_FAST   default: the reference's delay indices and phase arguments
 *                 bit for bit, the rest with FMA and the receive phasor
 *                 applied once per channel (~1e-7 relative L2 from the
 *                 reference);
 *   USX_BF_EXACT  every operation in the reference's order without
 *                 contraction (agrees to the last ulp of sincosf/cosf). */
enum { USX_BF_FAST = 0, USX_BF_EXACT = 1 };
int usx_cu_bf_plan_set_precision(usx_bf_plan* plan, int precision);

/* Launch shapes of the fast delay-and-sum (no counterpart in the reference):
 * variant i has a channel group (channels whose transmit geometry is shared
 * per event), a tile of tile_lines lateral lines x 32 depths per CTA and a
 * register cap for min_blocks resident CTAs per SM. All variants produce
 * bit-identical frames. usx_cu_bf_plan_autotune beamforms `data` once per
 * variant (plus a warm-up) `repeats` times, keeps the fastest in the plan,
 * writes every variant's mean milliseconds to ms_out[variant] (host, may be
 * NULL; usx_cu_bf_variant_count() entries), leaves the frame of the chosen
 * variant in `frame` and synchronises. Variant 0 is the default. */
int usx_cu_bf_variant_count(void);
int usx_cu_bf_variant_info(int index, int* channel_group, int* tile_lines, int* min_blocks, int* warp_lines);
/* The order in which variant i dispatches its CTA tiles: *deep_first = 1 when
 * every line group's deepest depth tile goes first (the lightest tiles form
 * the grid's tail), 0 for depth tiles in ascending order. */
int usx_cu_bf_variant_order(int index, int* deep_first);
/* The kernel family of variant i: 0 thread per pixel with channel groups
 * (tile_lines x 32 pixels per CTA), 1 the same with the trace windows staged
 * by bulk copies, 2 a transmit table (32 pixels per CTA, warp_lines lines x
 * 32 / warp_lines depths, one warp per channel_group channels; the transmit
 * delay, phasor and illumination weight computed once per pixel and event),
 * 3 the staged windows in a ring of shared-memory stages filled by a producer
 * warp (bulk copies on mbarriers, no CTA-wide barrier in the loop), 4
 * channel warps beside the pixel warps with the transmit terms tabulated per
 * pixel and event (the minimum-variance export, and the sums with the
 * channel combine in shared memory, in ascending channel order).
 * Families 1-4 fall back to variant 0 where they do not apply (RF data,
 * incoherent compounding; families 1 and 3 also need plane waves, family 2
 * at most 256 channels). */
int usx_cu_bf_variant_kind(int index, int* kind);
int usx_cu_bf_plan_set_variant(usx_bf_plan* plan, int index);
int usx_cu_bf_plan_get_variant(const usx_bf_plan* plan, int* index);
int usx_cu_bf_plan_autotune(usx_bf_plan* plan, const void* data, float* frame, int repeats, float* ms_out);

/* Minimum-variance solver of a plan (no counterpart in the reference, whose
 * one solver is combine_mv_windowed, beamformer.cpp:137-214):
 *   USX_MV_EXACT       FP32, the reference's operation order (default);
 *   USX_MV_TENSOR      BF16 covariance on the tensor cores with FP32
 *                      accumulation (full frames: a batched Hermitian rank-K
 *                      update on tcgen05, accumulators in tensor memory),
 *                      FP32 Cholesky, one refinement step against the FP32
 *                      covariance, FP64 re-solve where the refined residual
 *                      fails;
 *   USX_MV_TENSOR_MMA  the same with the covariance formed by warp-level
 *                      mma.sync inside the solve kernel;
 *   USX_MV_FP32        FP32 covariance formed inside the solve kernel from
 *                      the range rows by the lag recurrence (each entry
 *                      from its diagonal predecessor with 2 products per
 *                      range row instead of K), FP32 Cholesky and one solve:
 *                      the reference's precision, summed in another order.
 * Results agree within 1e-3 relative L2. */
enum { USX_MV_EXACT = 0, USX_MV_TENSOR = 1, USX_MV_TENSOR_MMA = 2, USX_MV_FP32 = 3 };
int usx_cu_bf_plan_set_mv_mode(usx_bf_plan* plan, int mode);
/* Counts since the last call (synchronises): pixels re-solved in FP64 and
 * pixels whose factorisation failed (these take the DAS sum). */
int usx_cu_bf_plan_mv_stats(usx_bf_plan* plan, int64_t* fp64_resolves,
                            int64_t* factorization_failures);

/* ------------------------------------------------- learned minimum variance */

/* The learned minimum variance has no counterpart in the reference; the
 * method it stands in for is the reference's minimum variance
 * (combine_mv_windowed, beamformer.cpp:137-214), which stays its per-pixel
 * fallback.
 *
 * A plan whose config has combiner USX_COMB_LEARNED_MV runs, per pixel:
 * the receive-delayed, compounded channel samples (rectangular apodisation,
 * as for minimum variance); 256 scale- and phase-free features (normalised
 * diagonal sums of the spatially smoothed covariance, the subarray-averaged
 * snapshot, L and the active aperture); the network (256 -> ... -> 128); the
 * predicted weights w~ = out / L, i < L; the distortionless residual
 * |1^H w~ - 1|. Pixels above `gate` are solved by the tensor-core minimum
 * variance; the others output n_act * (w~^H a) / conj(1^H w~), a the
 * subarray-averaged snapshot. Pixels with fewer than 4 active channels give
 * the DAS sum, as in the reference. Coherent and select compounding only.
 * The network is not owned and must outlive the plan's executions. */
int usx_cu_bf_plan_set_learned(usx_bf_plan* plan, usx_mlp* mlp, float gate);
/* How the learned path uses the network's weights w~ of a pixel that passes
 * the gate (no counterpart in the reference):
 *   n_beams < 0      as predicted (the default), the output above;
 *   n_beams = 0,2,4,6  the Capon problem of the reference's minimum variance,
 *                    min w^H (R + eps I) w subject to 1^H w = 1, solved
 *                    exactly within span{1, w~, e^{+-j 2 pi b i / L} for
 *                    b = 1..n_beams/2} through the pixel's snapshots (the
 *                    covariance is never formed). Equal to the exact minimum
 *                    variance when w~ is the Capon direction; always
 *                    distortionless. */
int usx_cu_bf_plan_set_learned_refine(usx_bf_plan* plan, int n_beams);
/* The refinement's second gate and its ablation (no counterpart in the
 * reference). With y = L^-1 Q^H 1 from the factor of the subspace system,
 * the subspace's Capon output power is 1/|y|^2 and that of the DFT beams
 * alone 1/|y_beams|^2, so s = |y_net|^2 / |y|^2 is the share of the output
 * power the network's direction removed. A pixel whose s exceeds
 * max_network_share goes to the exact minimum variance (its optimum lies well
 * outside the beams' span). use_network = 0 solves within the beams alone.
 * Defaults: use_network = 1, max_network_share = +inf (no second gate). */
int usx_cu_bf_plan_set_learned_subspace(usx_bf_plan* plan, int use_network, float max_network_share);
/* The refinement's third gate (no counterpart in the reference): a pixel
 * whose covariance trace tr(R) exceeds max_level_ratio times its depth's
 * level, the geometric mean of tr(R) over the frame's lateral lines at that
 * depth, goes to the exact minimum variance. Strong point targets raise tr(R)
 * far above the speckle level around them, where minimum variance forms deep
 * nulls that the refinement's subspace cannot. Default +inf (off); >= 1. */
int usx_cu_bf_plan_set_learned_level_gate(usx_bf_plan* plan, float max_level_ratio);
/* The level gate's neighbourhood: a pixel goes to the exact minimum variance
 * when any pixel within +/- half_lines lateral lines and +/- half_depths
 * depths exceeds its own depth's level by the gate, so that the flanks of a
 * strong target's response are solved with its peak. Default 0, 0 (the pixel
 * itself); each in [0, 16]. */
int usx_cu_bf_plan_set_learned_level_window(usx_bf_plan* plan, int half_lines, int half_depths);
/* Pixels gated to the exact solver and pixels beamformed by the learned path
 * since the last call (synchronises). */
int usx_cu_bf_plan_learned_stats(usx_bf_plan* plan, int64_t* gated, int64_t* pixels);
/* Training pairs from a coherent minimum-variance plan in USX_MV_TENSOR mode:
 * every execution also writes, per pixel row r = frame * n_pix + pix,
 * features[r][256], weights[r][128] = L w_i / sum(w) interleaved (re, im),
 * zero for i >= L, and valid[r] = 1 where a Capon solve exists (0 for the
 * DAS rule and failed factorisations). Device buffers; NULLs turn it off. */
int usx_cu_bf_plan_set_training_export(usx_bf_plan* plan, float* features, float* weights,
                                       uint8_t* valid);

/* The network: fully connected layers dims[0] -> dims[1] -> ... ->
 * dims[n_layers], ReLU between layers, FP32 master weights with a BF16 copy
 * for the GEMMs (BF16 operands, FP32 accumulation: tcgen05 with the
 * accumulator in tensor memory for the forward layers of width 128 or 256
 * whose input width is a multiple of 64, mma.sync for the rest and for the
 * backward pass). Every width must be a
 * positive multiple of 128. Parameters are laid out per layer as W_l
 * [dims[l]][dims[l+1]] row-major followed by b_l [dims[l+1]]. Weights start
 * He-uniform from `seed`, biases at zero. */
int usx_cu_mlp_create(usx_ctx* ctx, int n_layers, const int* dims, uint64_t seed, usx_mlp** out);
int usx_cu_mlp_destroy(usx_mlp* mlp);
int usx_cu_mlp_num_params(const usx_mlp* mlp, int64_t* count);
/* FP32 parameters to / from host memory (synchronises). */
int usx_cu_mlp_get_params(usx_mlp* mlp, float* host);
int usx_cu_mlp_set_params(usx_mlp* mlp, const float* host);
/* y[rows][dims[n_layers]] = net(x[rows][dims[0]]), FP32 device buffers. */
int usx_cu_mlp_forward(usx_mlp* mlp, const float* x, int64_t rows, float* y);
/* One training step on device buffers x[rows][dims[0]], target and mask
 * [rows][dims[n_layers]] (mask may be NULL): gradients of
 * sum(mask * (y - target)^2) / (rows * dims[n_layers]), then, when lr > 0,
 * one Adam step (beta 0.9, 0.999, eps 1e-8). rows must be a multiple of 128.
 * loss_host and grad_host (n_params floats) are optional host outputs and
 * make the call synchronise. */
int usx_cu_mlp_train_step(usx_mlp* mlp, const float* x, const float* target, const float* mask,
                          int64_t rows, float lr, float* loss_host, float* grad_host);
/* Training loss of usx_cu_mlp_train_step:
 *   USX_MLP_LOSS_MSE         the masked mean squared error above (default);
 *   USX_MLP_LOSS_LMV_OUTPUT  for the learned minimum variance (256 -> 128):
 *     per row, with w the 64 predicted complex weights, t the target weights,
 *     a the normalised subarray-averaged snapshot (input features 128..255)
 *     and the mask selecting i < L, the squared error of the combiner output
 *     sum conj(w) a / conj(sum w) against the same with t, plus the squared
 *     distortionless residual |sum w / L - 1|^2, plus beta * sum mask
 *     |w - t|^2; the sum over rows divided by rows;
 *   USX_MLP_LOSS_LMV_SUBSPACE  for the learned-subspace refinement (256 -> 128):
 *     per row, with P the projector onto the complement of the DFT beams
 *     b = 0, +1, -1, +2, -2 of length L (the first min(5, L)), u = P w,
 *     v = P t: 1 - |u^H v|^2 / (|u|^2 |v|^2) (skipped where the target lies in
 *     the beams' span) plus beta * sum mask |w - t|^2 / L; summed over rows
 *     and divided by rows. */
enum { USX_MLP_LOSS_MSE = 0, USX_MLP_LOSS_LMV_OUTPUT = 1, USX_MLP_LOSS_LMV_SUBSPACE = 2 };
int usx_cu_mlp_set_loss(usx_mlp* mlp, int kind, float beta);
/* Forward GEMM of the network: USX_MLP_GEMM_AUTO (default) takes the tcgen05
 * GEMM wherever the layer's shape allows it, USX_MLP_GEMM_MMA_SYNC always the
 * mma.sync GEMM. Both accumulate the same BF16 products in FP32; they differ
 * only in the order of the additions. */
enum { USX_MLP_GEMM_AUTO = 0, USX_MLP_GEMM_MMA_SYNC = 1 };
int usx_cu_mlp_set_gemm_path(usx_mlp* mlp, int path);

/* Beamformer::beamform_sequence (reference beamformer.cpp:551-569) in one
 * launch: frame f uses the plan's events [first + f*events_per_frame,
 * first + (f+1)*events_per_frame) of the single acquisition `data`; frames
 * are written frame_stride complex apart. This is how a Doppler ensemble is
 * formed. */
int usx_cu_bf_execute_sequence(usx_bf_plan* plan, int events_per_frame, int n_frames,
                               const void* data, float* frames, int64_t frame_stride);

/* Frames of many plans in one persistent launch (reference: Beamformer::beamform,
 * beamformer.cpp:297-549, once per frame): entry i beamforms data[i] with
 * plans[i] into frames[i] (one frame each; any probe, grid, transmit set and
 * plain combiner — DAS, DMAS, coherence factor — coherent or select
 * compounding, all IQ or all RF). The CTAs take tiles of all entries from one
 * work counter, so frames of uneven size share the GPU without a tail per
 * frame; each frame equals its plan's own execution bit for bit. Up to 48
 * entries per launch (more are split); the plans must belong to ctx. */
int usx_cu_bf_execute_queue(usx_ctx* ctx, int n, usx_bf_plan* const* plans, const void* const* data,
                            float* const* frames);

/* One-shot convenience: plan, execute, destroy (not graph-capturable). */
int usx_cu_beamform(usx_ctx* ctx, const usx_channel_desc* cd, const void* data,
                    const usx_grid_desc* grid, const float* points_host,
                    const usx_beamformer_config* cfg, int event_begin, int event_end,
                    float* frame);

/* ------------------------------------------------------------- post-process */

/* envelope (postprocess.cpp:67-82): |z| when fdem > 0, else the modulus of
 * the analytic signal of the real part along axis 1 (radix-2 FFT Hilbert). */
int usx_cu_envelope(usx_ctx* ctx, const float* frame, int n0, int n1, float fdem, float* env);
/* apply_tgc (postprocess.cpp:84-98); points device [n0*n1][3]. */
int usx_cu_apply_tgc(usx_ctx* ctx, const float* env, int n0, int n1, const float* points,
                     float attenuation_db_cm_mhz, float center_frequency_hz, float* out);
/* log_compress (postprocess.cpp:100-117); reference <= 0 uses the maximum
 * (found on the device). */
int usx_cu_log_compress(usx_ctx* ctx, const float* env, int64_t n, float dynamic_range_db,
                        float gain_db, float reference, float* out);
/* Maximum of a float array (device) into *out_host (synchronises). */
int usx_cu_max(usx_ctx* ctx, const float* x, int64_t n, float* out_host);
/* scan_convert (postprocess.cpp:119-178). `grid` gives type, axes (host) and
 * apex; points device [n0*n1][3]; pixels device [height][width];
 * extent (host) receives x_min, x_max, z_min, z_max. */
int usx_cu_scan_convert(usx_ctx* ctx, const float* image, const usx_grid_desc* grid,
                        const float* points_host, int width, int height, float fill,
                        float* pixels, float* extent);

/* ------------------------------------------------------- Doppler / strain */

/* apply_wall_filter (doppler.cpp:51-75): ensemble [n_frames][n_pix] complex. */
int usx_cu_wall_filter(usx_ctx* ctx, const float* ens, int n_frames, int64_t n_pix, int type,
                       int order, float* out);
/* color_flow (doppler.cpp:77-176). Outputs device [n0*n1]; *nyquist (host). */
int usx_cu_color_flow(usx_ctx* ctx, const float* ens, int n_frames, int n0, int n1,
                      const float* axis1_host, float fdem, float prf, float speed_of_sound,
                      const usx_doppler_config* cfg, float* velocity, float* power,
                      float* variance, uint8_t* valid, float* nyquist);
/* Many colour-flow ensembles of uneven length in one launch sequence
 * (reference: color_flow per ensemble, doppler.cpp:77-176): ensemble e has
 * n_frames[e] frames starting at frame offset frame_offset[e] of `ens` (all
 * the same grid); outputs are [n_ens][n0*n1], each map bit for bit what
 * usx_cu_color_flow gives for that ensemble. One wall-filter and one flow
 * launch per 64 ensembles (fewer when many distinct lengths share a call),
 * then one power-gate launch for all; n_ens <= 65535. */
int usx_cu_color_flow_batch(usx_ctx* ctx, const float* ens, int n_ens, const int* n_frames_host,
                            const int64_t* frame_offset_host, int n0, int n1,
                            const float* axis1_host, float fdem, float prf,
                            float speed_of_sound, const usx_doppler_config* cfg, float* velocity,
                            float* power, float* variance, uint8_t* valid);
/* Colour flow that allocates nothing. No counterpart in the reference: this
 * is for callers that cannot allocate device memory while they run (a
 * real-time acquisition loop with a fixed memory budget, or a host that owns
 * the device allocator and only lends this library a stream). It computes
 * exactly what usx_cu_color_flow computes, on `stream` (a cudaStream_t; NULL is the legacy default stream)
 * instead of a context, with its working memory in a fixed array that every
 * device loading this library reserves until the process exits.
 *   Limit: n_frames * n0 * n1 <= 1048576 complex samples (8 MiB of scratch);
 *   larger ensembles return USX_ERR_INVALID (use usx_cu_color_flow).
 *   The first call on each device looks the array up (cudaGetSymbolAddress);
 *   make that first call before capturing the stream into a graph.
 *   All calls share the one array: calls whose work overlaps on the GPU (on
 *   different streams, or from different threads) race and must be
 *   serialised by the caller. */
int usx_cu_color_flow_noalloc(void* stream, const float* ens, int n_frames, int n0, int n1,
                              const float* axis1_host, float fdem, float prf, float speed_of_sound,
                              const usx_doppler_config* cfg, float* velocity, float* power,
                              float* variance, uint8_t* valid, float* nyquist);
/* power_doppler (doppler.cpp:178-186). */
int usx_cu_power_doppler(usx_ctx* ctx, const float* ens, int n_frames, int64_t n_pix, int type,
                         int order, float* power);
/* estimate_axial_displacement (doppler.cpp:188-273). */
int usx_cu_axial_displacement(usx_ctx* ctx, const float* before, const float* after, int n0,
                              int n1, const float* axis1_host, float fdem, float speed_of_sound,
                              int kernel_axial, int kernel_lateral, int max_lag, float* axial,
                              float* correlation);
/* axial_strain (doppler.cpp:275-305). */
int usx_cu_axial_strain(usx_ctx* ctx, const float* axial, int n0, int n1,
                        const float* axis1_host, int fit_length, float* strain);

#ifdef __cplusplus
}
#endif

#endif /* USX_CU_H */
