/* usx_types.h — plain-old-data descriptors shared by the C-ABI (usx_cu.h) and
 * the CPU oracle.
 *
 * Every struct mirrors one of the reference's C++ value types field for field,
 * with the same defaults (documented beside each field) and the same units
 * (SI: metres, seconds, hertz). Enumerations keep the reference's numeric
 * values so that a caller can cast its own enum straight across the boundary.
 *
 * Reference types mirrored (core/include/usx/...):
 *   usx_probe              types.hpp:68-91      (Probe)
 *   usx_medium             types.hpp:103-109    (Medium)
 *   usx_acquisition        types.hpp:114-134    (Acquisition)
 *   usx_transmit           types.hpp:157-173    (Transmit)
 *   usx_beamformer_config  beamformer.hpp:66-106 (BeamformerConfig)
 *   usx_demod_config       demodulate.hpp:23-40  (DemodConfig)
 *   usx_simulator_config   simulator.hpp:77-116  (SimulatorConfig)
 *   usx_doppler_config     doppler.hpp:41-74     (DopplerConfig)
 */
#ifndef USX_TYPES_H
#define USX_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* TransmitType (types.hpp:157) */
enum { USX_TX_FOCUSED = 0, USX_TX_PLANE_WAVE = 1, USX_TX_DIVERGING = 2 };
/* GridType (types.hpp:234) */
enum { USX_GRID_CARTESIAN = 0, USX_GRID_SECTOR = 1 };
/* Window (types.hpp:289) */
enum { USX_WIN_RECT = 0, USX_WIN_HANN = 1, USX_WIN_HAMMING = 2, USX_WIN_TUKEY = 3, USX_WIN_BLACKMAN = 4 };
/* Combiner (beamformer.hpp:42-46); USX_COMB_LEARNED_MV has no reference counterpart. */
enum { USX_COMB_DAS = 0, USX_COMB_DMAS = 1, USX_COMB_MV = 2, USX_COMB_LEARNED_MV = 3 };
/* Compounding (beamformer.hpp:49-64) */
enum { USX_COMP_COHERENT = 0, USX_COMP_INCOHERENT = 1, USX_COMP_SELECT = 2 };
/* WallFilter (doppler.hpp:29-39) */
enum { USX_WALL_NONE = 0, USX_WALL_POLYNOMIAL = 1, USX_WALL_MEAN = 2 };

typedef struct usx_probe {
  int32_t n_elements;       /* 128 */
  float pitch;              /* 300e-6 m */
  float element_width;      /* 270e-6 m */
  float elevation_height;   /* 5e-3 m */
  float center_frequency;   /* 5e6 Hz */
  float bandwidth;          /* 0.6 fractional */
} usx_probe;

typedef struct usx_medium {
  float speed_of_sound;     /* 1540 m/s */
  float attenuation;        /* 0.5 dB/(cm MHz), one way */
  float density;            /* 1000 kg/m^3 (unused) */
} usx_medium;

typedef struct usx_acquisition {
  float sampling_frequency; /* 40e6 Hz */
  int32_t n_samples;        /* 2048 */
  float t0;                 /* 0 s */
  float prf;                /* 5000 Hz */
} usx_acquisition;

/* One transmit event. `delays` and `apodization` are HOST arrays of
 * probe.n_elements floats, or NULL for an empty vector (reference semantics:
 * an empty apodization means every element fires with weight 1). */
typedef struct usx_transmit {
  int32_t type;             /* USX_TX_* (default plane wave) */
  float angle;              /* rad */
  float focus[3];           /* m, default (0,0,0.03) */
  float origin[3];          /* m */
  const float* delays;
  const float* apodization;
} usx_transmit;

/* The metadata half of ChannelData (types.hpp:187-217); the samples are passed
 * separately as a device pointer laid out [event][channel][sample], either
 * float (RF) or interleaved complex float (IQ). */
typedef struct usx_channel_desc {
  usx_probe probe;
  usx_medium medium;
  usx_acquisition acq;
  int32_t n_events;
  const usx_transmit* transmits;   /* host array of n_events */
  int32_t is_iq;
  float demodulation_frequency;
} usx_channel_desc;

typedef struct usx_grid_desc {
  int32_t type;             /* USX_GRID_* */
  int32_t n_axis0;          /* lateral / theta */
  int32_t n_axis1;          /* depth / range, fastest */
  float apex[3];
  const float* axis0;       /* host, n_axis0 */
  const float* axis1;       /* host, n_axis1 */
} usx_grid_desc;

typedef struct usx_beamformer_config {
  float f_number;              /* 1.75 */
  int32_t rx_window;           /* USX_WIN_HANN */
  float tukey_alpha;           /* 0.5 */
  int32_t combiner;            /* USX_COMB_DAS */
  int32_t compounding;         /* USX_COMP_COHERENT */
  int32_t transmit_weighting;  /* 1 */
  int32_t coherence_factor;    /* 0 */
  int32_t mv_subarray;         /* 16 */
  float mv_diagonal_loading;   /* 1e-2 */
  int32_t mv_range_average;    /* 2 */
} usx_beamformer_config;

typedef struct usx_demod_config {
  float demodulation_frequency; /* 0 -> probe centre frequency */
  float cutoff_fraction;        /* 0.5 */
  int32_t filter_taps;          /* 33 */
  int32_t decimation;           /* 1 */
} usx_demod_config;

typedef struct usx_simulator_config {
  float pulse_cycles;            /* 2.5 (unused when bandwidth > 0) */
  int32_t tx_window;             /* USX_WIN_HANN */
  float tx_f_number;             /* 2.0 */
  int32_t oversampling;          /* 4 */
  int32_t full_transmit_diffraction; /* 1 */
  float incident_trim_db;        /* -40 */
  float max_incident_window_us;  /* 30 */
  int32_t apply_attenuation;     /* 1 */
  int32_t apply_directivity;     /* 1 */
  int32_t apply_spreading;       /* 1 */
  float noise_db;                /* -60 */
  uint32_t noise_seed;           /* 7 */
  int32_t enable_motion;         /* 1 */
} usx_simulator_config;

typedef struct usx_doppler_config {
  int32_t wall_filter;           /* USX_WALL_POLYNOMIAL */
  int32_t polynomial_order;      /* 1 */
  int32_t loupas;                /* 1 */
  int32_t kernel_axial;          /* 4 */
  int32_t kernel_lateral;        /* 1 */
  float power_threshold_db;      /* -35 */
  float coherence_threshold;     /* 0.35 */
} usx_doppler_config;

/* A point scatterer, as the simulator consumes it: position, amplitude and
 * velocity packed into 8 floats (the last is padding) so that one scatterer is
 * two aligned 16-byte loads. Reference: Scatterer, simulator.hpp:28-32. */
typedef struct usx_scatterer {
  float x, y, z, amplitude;
  float vx, vy, vz, pad;
} usx_scatterer;

#ifdef __cplusplus
}
#endif

#endif /* USX_TYPES_H */
