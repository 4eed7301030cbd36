/* usx_oracle.h — CPU oracle for the usx imaging path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * engine's algorithms (AadithyaSairam/ultrasound-engine, core/src/ sources), used
 * as the checker for the CUDA kernels and as the timed CPU baseline. Nothing in
 * the product links or calls it; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it.
 *
 * Every function exists twice: `_f32` follows the reference's float arithmetic
 * operation by operation (no FMA contraction, same evaluation order, same libm
 * calls), so it reproduces the reference C++ to the last bit or ulp; `_f64`
 * runs the same algorithm in double precision and is the FP64 oracle that
 * FP32 errors are reported against.
 *
 * Complex data is interleaved (re, im). Array layouts follow the reference:
 * channel data [event][channel][sample], frames [axis0][axis1] with axis1
 * fastest, grid points [pixel][x,y,z].
 */
#ifndef USX_ORACLE_H
#define USX_ORACLE_H

#include "../include/usx_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_DECL(R, S)                                                                   \
  /* types.cpp:126-148 */                                                                \
  R orc_window_value_##S(int window, R u, R tukey_alpha);                                 \
  /* geometry.cpp:111-121 */                                                             \
  R orc_element_directivity_##S(R element_width, R wavelength, R sin_theta);             \
  /* demodulate.cpp:13-34; returns the tap count written to h (h holds >= n_taps+1) */   \
  int orc_design_lowpass_##S(int n_taps, R normalized_cutoff, R* h);                     \
  /* simulator.cpp:140-154; returns the tap count; p may be NULL to query */             \
  int orc_pulse_##S(const usx_probe* probe, const usx_acquisition* acq,                  \
                    const usx_simulator_config* cfg, R* p, R* half_duration);            \
  /* simulator.cpp:213-419. noise_z: n_events*n_ch*n_smp standard normals (the */        \
  /* draws of std::normal_distribution seeded per event) or NULL for no noise. */        \
  int orc_simulate_##S(const usx_channel_desc* cd, const usx_simulator_config* cfg,      \
                       const usx_scatterer* scat, long n_scat, const float* noise_z,     \
                       R* rf);                                                           \
  /* demodulate.cpp:36-121; iq has n_events*n_ch*ceil(n/dec) complex samples */          \
  int orc_demodulate_##S(const usx_channel_desc* cd, const usx_demod_config* cfg,        \
                         const R* rf, R* iq);                                            \
  /* beamformer.cpp:297-549; data is RF (real) or IQ (interleaved complex) per cd */     \
  int orc_beamform_##S(const usx_channel_desc* cd, const R* data, int n_pix_axis0,       \
                       int n_pix_axis1, const float* points,                             \
                       const usx_beamformer_config* cfg, int event_begin, int event_end, \
                       R* frame);                                                        \
  /* learned minimum variance (no reference counterpart): MV beamform plus per-pixel */ \
  /* features [n_pix][256], Capon weights L w / sum(w) [n_pix][128] and valid flags */     \
  /* Learned-subspace refinement in the MV combiner (NULL disables). */    \
  void orc_set_lmv_subspace_##S(const float* net_out128, int n_beams);     \
  int orc_mv_training_pairs_##S(const usx_channel_desc* cd, const R* data, int n_pix_axis0, \
                                int n_pix_axis1, const float* points,                     \
                                const usx_beamformer_config* cfg, R* frame, R* feat,      \
                                R* weights, unsigned char* valid);                        \
  /* beamformer.cpp:249-295 */                                                           \
  R orc_transmit_sensitivity_##S(const usx_probe* probe, const usx_transmit* tx,         \
                                 const float* point, R wavelength);                      \
  /* geometry.cpp:82-109 */                                                              \
  R orc_transmit_arrival_time_##S(const usx_transmit* tx, const float* point, R c);      \
  /* doppler.cpp:15-47; M is n*n */                                                      \
  void orc_polynomial_reject_matrix_##S(int n, int order, R* M);                         \
  /* doppler.cpp:51-75; ens/out: n_frames*n_pix complex */                               \
  int orc_wall_filter_##S(const R* ens, int n_frames, long n_pix, int type, int order,   \
                          R* out);                                                       \
  /* doppler.cpp:77-176 */                                                               \
  int orc_color_flow_##S(const R* ens, int n_frames, int n0, int n1, const float* axis1, \
                         float fdem, R prf, R c, const usx_doppler_config* cfg,          \
                         R* velocity, R* power, R* variance, unsigned char* valid,       \
                         R* nyquist);                                                    \
  /* doppler.cpp:178-186 */                                                              \
  int orc_power_doppler_##S(const R* ens, int n_frames, long n_pix, int type, int order, \
                            R* power);                                                   \
  /* doppler.cpp:188-273 */                                                              \
  int orc_axial_displacement_##S(const R* before, const R* after, int n0, int n1,        \
                                 const float* axis1, float fdem, R c, int kernel_axial,  \
                                 int kernel_lateral, int max_lag, R* axial, R* corr);    \
  /* doppler.cpp:275-305 */                                                              \
  int orc_axial_strain_##S(const R* axial, int n0, int n1, const float* axis1,           \
                           int fit_length, R* strain);                                   \
  /* postprocess.cpp:67-82; frame complex interleaved */                                 \
  int orc_envelope_##S(const R* frame, int n0, int n1, float fdem, R* env);              \
  /* postprocess.cpp:47-65 */                                                            \
  int orc_analytic_##S(const R* data, int n0, int n1, R* out);                           \
  /* postprocess.cpp:84-98 */                                                            \
  int orc_apply_tgc_##S(const R* env, int n0, int n1, const float* points, R atten,      \
                        R f0, R* out);                                                   \
  /* postprocess.cpp:100-117 */                                                          \
  int orc_log_compress_##S(const R* env, long n, R dr_db, R gain_db, R reference,        \
                           R* out);                                                      \
  /* postprocess.cpp:119-178; extent: x_min, x_max, z_min, z_max */                     \
  int orc_scan_convert_##S(const R* image, int grid_type, int n0, int n1,                \
                           const float* axis0, const float* axis1, const float* apex,    \
                           const float* points, int width, int height, R fill,           \
                           R* pixels, R* extent);

ORC_DECL(float, f32)
ORC_DECL(double, f64)

/* Number of OpenMP threads the oracle will use (1 when built without OpenMP). */
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif /* USX_ORACLE_H */
