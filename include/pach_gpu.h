/*
 * pach_gpu.h -- C ABI of the GB300 (sm_103a) stochastic split ray tracer.
 *
 * Drop-in boundary for Pachyderm's SplitRayTracer path.  A host (the C# Simulation_Type shim
 * through P/Invoke, the C++ mirror in split_ray_tracer.hpp, or Python through ctypes) passes plain
 * arrays; the library owns every device allocation and handle.  Plain C types only.
 *
 * Reference interfaces replaced (paths relative to Pachyderm_Acoustic_Universal/; "TaskAll" is
 * "Classes_Complete_Trace - TaskAll.cs"):
 *   pach_scene_create        Polygon_Scene ctor + Construct + partition
 *                            (Classes_Scenes.cs:70-105, 447-630, 727-755)
 *   pach_trace_begin         SplitRayTracer ctor + Begin (TaskAll:68-177, 209-240)
 *   pach_trace_poll          ThreadState / ProgressMsg (TaskAll:246-250, 742-763)
 *   pach_trace_cancel        Conclude_Simulation / cancellation token (TaskAll:252-255, 276-280)
 *   pach_trace_wait          the host's poll-until-stopped loop
 *   pach_trace_get_histograms Combine_ThreadLocal_Results + Receiver_Bank histogram getters
 *                            (TaskAll:768-774; Classes_Receivers.cs:676-679, 924-927, 1088-1102, 1774-1786)
 *   pach_trace_get_stats     PercentLost, _currentRay, _rayTotal, _ts (TaskAll:40-47, 776-782)
 *   pach_medium_properties   Uniform_Medium ctor (Classes_Medium_Props.cs:286-299)
 *   pach_medium_attenuation_third_octave  Calculate_Attenuation, third octaves (Classes_Medium_Props.cs:51-89)
 *   pach_math_*              AcousticalMath (Classes_Math.cs:272-586, 934-1005)
 *   pach_direct_sound        Direct_Sound, point sources (Classes_Direct.cs:654-685, 772-823)
 *   pach_trace_get_map       PachMapReceiver as the run's Receiver_Bank (Pach_Map_Receiver.cs:34-1834)
 *   pach_map_parameters, pach_etc_parameters  Get_RT_Map / Get_EDT_Map / Get_Clarity_Map /
 *                            Get_Definition_Map without coherent superposition (Pach_Map_Receiver.cs:925-1270)
 *
 * Error behaviour: every entry point returns a pach_status; the message of the last failure on
 * the calling thread is available from pach_last_error.  No callbacks and no C++ exceptions cross
 * the ABI (a failed host allocation returns PACH_ERR_OUT_OF_MEMORY).
 */
#ifndef PACH_GPU_H
#define PACH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PACH_ABI_VERSION 2
#define PACH_BANDS 8

typedef enum {
    PACH_OK = 0,
    PACH_ERR_INVALID_ARGUMENT = 1,
    PACH_ERR_OUT_OF_MEMORY = 2,
    PACH_ERR_CUDA = 3,
    PACH_ERR_TIMEOUT = 4,          /* pach_trace_wait ran out of time; the run continues */
    PACH_ERR_CANCELLED = 5,
    PACH_ERR_BOUNDS = 6,           /* a device queue or stack bound was exceeded */
    PACH_ERR_NOT_READY = 7,
    PACH_ERR_NO_DEVICE = 8,
    PACH_ERR_GAVE_UP = 9           /* a bounded device wait or work cap ran out */
} pach_status;

typedef enum { PACH_RUN_RUNNING = 0, PACH_RUN_STOPPED = 1, PACH_RUN_FAILED = 2, PACH_RUN_CANCELLED = 3 } pach_run_state;

typedef enum {
    PACH_SOURCE_GEODESIC = 0,      /* GeodesicSource: order-1 icosphere face (ray mod 80) + random point */
    PACH_SOURCE_RANDOM = 1,        /* RandomSource: theta, phi ~ U[0, 2pi) */
    PACH_SOURCE_UNIFORM = 2        /* uniform on the sphere */
} pach_source_kind;

/* Scene: polygons over a shared vertex list (any vertex count; fan-triangulated, polygon id kept),
 * 8-band absorption / scattering / transmission per polygon, and the air state of the Scene ctor. */
typedef struct {
    int32_t n_vertices;
    const double *vertices;        /* [3*n_vertices] metres */
    int32_t n_polys;
    const int32_t *poly_offsets;   /* [n_polys+1] into poly_indices */
    const int32_t *poly_indices;
    const double *absorption;      /* [n_polys*8] */
    const double *scattering;      /* [n_polys*8] */
    const double *transmission;    /* [n_polys*8] or NULL */
    double temp_c;                 /* degC */
    double rel_humidity;           /* percent */
    double pressure_hpa;           /* hPa, as the Scene ctor (1013.25 = 101.325 kPa) */
    int32_t air_choice;            /* 0 ISO 9613-1, 1 Evans-Bazley, 2 tables */
    int32_t edge_correction;
    int32_t bvh_leaf_max;          /* triangles per BVH leaf at most (1..8); 0 = default (3) */
    int32_t reserved1;
} pach_scene_desc;

typedef struct {
    double origin[3];
    double power_db[PACH_BANDS];   /* dB re 1e-12 W per octave band */
    int32_t kind;                  /* pach_source_kind */
    int32_t reserved;
} pach_source_desc;

typedef struct {
    double origin[3];
    double radius;                 /* Spherical_Receiver.Radius (the reference ctor fixes 1 m) */
} pach_receiver_desc;

typedef struct {
    uint64_t seed;                 /* Philox key; a run is reproducible for a fixed seed */
    int64_t ray_count;             /* primary rays (SplitRayTracer rayCount > 0); < 1: convergence mode as
                                      the reference's rayCount < 1 (TaskAll:111-176, 300-330): revolutions of
                                      80 primaries per source until the convergence checks of two receivers
                                      (the farthest the source sees, the farthest it does not) agree --
                                      0: SpecMin_Convergence_Check, < 0: Minimum_Convergence_Check */
    int64_t ray_begin;             /* index of the first primary: a shard [ray_begin, ray_begin+ray_count)
                                      draws the same random streams as in an unsharded run */
    double cutoff_length_m;        /* SplitRayTracer "cutoffTime" argument: a LENGTH, COTime = L / c */
    int32_t oct_lo, oct_hi;        /* octave range, inclusive, 0 = 62.5 Hz .. 7 = 8 kHz */
    int32_t is_order;              /* image-source order already covered; -1: rays also record the direct path */
    int32_t sample_rate;           /* histogram rate Hz (Receiver_Bank SampleRate, 1000 for 1 ms bins) */
    double hist_cotime_ms;         /* histogram length ms (Receiver_Bank COTime_in) */
    int32_t pure_specular;         /* 1: all scattering and transmission forced to 0 */
    int32_t max_broadband_bounces; /* 0 = derived bound from the scene's least lossy surface */
    int64_t max_segments_per_ray;  /* safety cap on one octave ray (0 = 1<<22) */
    int64_t feed_batch;            /* primaries handed to the device per phase-A launch (0 = default) */
    int32_t block_threads;         /* threads per block of the trace and shade kernels; 0 = default */
    int32_t blocks_per_sm;         /* resident blocks per SM to launch; 0 = occupancy maximum */
    int32_t wave_kilo_items;       /* octave rays per wave, in units of 1024; 0 = default (8192) */
    int32_t ring_log2;             /* ring queue capacity 2^ring_log2 octave rays; 0 = default (2^22..2^28 by
                                      the run's primaries, 2048 rays each) */
    int32_t kernel_timing;         /* 1: CUDA events around every kernel (per-kernel times in pach_stats) */
    int32_t ray_sort;              /* 1: order each wave by (direction octant, origin cell) before tracing;
                                      0 = default (off: measured +6 % walk rate in the 20k-triangle
                                      hall, less than the sort costs) */
    int32_t traversal;             /* BVH walk: 0 = default, 1 = one leaf at a time, 2 = speculative
                                      (lanes holding a leaf keep descending until the whole warp holds
                                      one, then the warp tests its leaves together), 3 = in the shading
                                      kernel (no separate walk pass; the default up to 64 triangles) */
    int32_t capture;               /* 1: record energy per receiver, time window and emission-direction
                                      bin; 2: per primary, receiver and time window
                                      (pach_trace_get_capture, pach_proposal.h) */
    const double *prim_dirs;       /* optional [ray_count][3] emission directions (importance sampling) */
    const double *prim_weights;    /* optional [ray_count] emission weights (1/q) */
    const float *proposal;         /* optional [n_proposal][160] learned-proposal lobes (pach_proposal.h) */
    int32_t n_proposal;
    int32_t bvh_format;            /* BVH nodes the trace kernel walks: 0 = default, 1 = 128-byte float
                                      boxes, 2 = 48-byte nodes with 8-bit child boxes (scenes whose
                                      triangle ids fit 24 bits; others walk the float boxes) */
    double proposal_mix;           /* weight of uniform emission in the proposal, (0, 1]; 0 = 0.3 */
    double capture_edges_ms[3];    /* capture windows, ms after the direct arrival; zeros = 80, 400, 1200 */
    const struct pach_map_desc *map; /* optional mapping receivers (single-room runs), else NULL */
    int64_t max_rays;              /* convergence mode (ray_count < 1): primaries traced at most before the run
                                      stops unconverged (0 = 2^24) */
} pach_trace_params;

/* Mapping receivers (PachMapReceiver, Pach_Map_Receiver.cs:34-1834): many small spheres, typically one
 * per face or vertex of an audience mesh, found along each segment by a walk over a uniform grid of
 * cells 4 x 4 x 2.5 increments.  Detection as Map_Receiver.CheckRay / CheckBroadbandRay
 * (Pach_Map_Receiver.cs:1780-1826): energy I 10^(-0.1 m t) / (pi r^2) with t the arrival time in
 * seconds AFTER the receiver's direct arrival (the reference's exponent takes that time, not a
 * distance), no chord-length weight, 1 ms bins counted from the direct arrival, every band of a
 * broadband ray.  The direct arrival is |source - receiver| / c for a single source and 0 for a
 * cluster (Map_Receiver ctor, Pach_Map_Receiver.cs:1737-1751). */
typedef struct pach_map_desc {
    int32_t n_receivers;
    int32_t time_1pt;              /* 1: one bin per band holding every arrival (Histogram_1Pt) */
    const double *origins;         /* [3*n_receivers] sphere centres (PachMapReceiver.Partition places them) */
    double increment;              /* sphere DIAMETER, m (radius = increment / 2) */
    double cutoff_ms;              /* histogram length: (int)(cutoff_ms / 1000 * 1000) bins of 1 ms */
    int32_t walk;                  /* 0: the grid walks as the reference writes them (the broadband walk steps
                                      by the sign of the ray's POSITION and stops when any cell index reaches
                                      the end cell's; the octave walk never visits the end cell);
                                      1: every cell the segment crosses, end cell included */
    int32_t directional;           /* 1: Directional_Histogram per receiver (pressure sqrt(E rho c), +-x/y/z
                                      arrival components; pach_trace_get_map_directions) */
} pach_map_desc;

/* One room of a batch run (pach_batch_begin). */
typedef struct {
    const struct pach_scene *scene;
    const pach_source_desc *sources;
    int32_t n_sources;
    int32_t n_receivers;
    const pach_receiver_desc *receivers;
    int64_t ray_count;             /* primary rays of this room */
    double cutoff_length_m;        /* this room's SplitRayTracer cutoff length */
} pach_room_desc;

typedef struct {
    int32_t state;                 /* pach_run_state */
    int32_t last_status;           /* pach_status of a failed run */
    int64_t rays_done;             /* _currentRay */
    int64_t rays_total;
    int64_t end_traces;            /* _rayTotal ("sub-rays") */
    int64_t segments;
} pach_progress;

typedef struct {
    int64_t primaries;
    int64_t segments;              /* shoot calls, broadband + octave, hit or miss */
    int64_t segments_broadband;
    int64_t segments_phase_b;
    int64_t segments_phase_c;
    int64_t octave_rays;
    int64_t end_traces;
    int64_t detections;
    int64_t capped;
    int64_t fp64_retests;          /* FP32 hits re-tested in FP64 (near edge / grazing) */
    int64_t queue_overflows;
    int64_t stack_spills;
    double lost_energy;            /* W (sum over rays, unscaled) */
    double initial_energy;
    double percent_lost;           /* 100 lost / initial (PercentLost) */
    int32_t h_oct;
    int32_t bins;
    double cotime_s;
    double sound_speed;
    double rho_c;
    double air_atten_db_per_m[PACH_BANDS];
    double device_ms;              /* CUDA-event time of all kernels of the run */
    double trace_ms;               /* per-kernel CUDA-event times (kernel_timing = 1, else 0) */
    double shade_ms;
    double broadband_ms;
    double sort_ms;
    int64_t waves;                 /* wavefront iterations that traced octave rays */
    int64_t kernel_launches;
    int64_t peak_live_rays;        /* most octave rays held in the ring at once */
    int64_t bvh_nodes_visited;     /* octave-ray traversal work: inner BVH nodes visited, and */
    int64_t tri_tests;             /* triangles tested (counted when kernel_timing = 1; else 0 on
                                      scenes walked by the speculative walk) */
    double wall_ms;
    int32_t accel[3];              /* BVH inner nodes, leaves, depth */
    int32_t walk;                  /* the walk used: BVH node bytes (48 or 128) + 1000 x traversal (1-3) */
    int64_t revolutions;           /* convergence mode: revolutions traced (primaries = revolutions x period) */
    int32_t converged;             /* convergence mode: 1 when the checks agreed, 0 when max_rays stopped it */
    int32_t check_receivers[2];    /* convergence mode: receivers of the two checks (-1: none) */
    int32_t reserved2;
} pach_stats;

typedef struct pach_scene pach_scene;
typedef struct pach_run pach_run;

const char *pach_version(void);
/* Copies the last error message of the calling thread; returns its length. */
int pach_last_error(char *buf, size_t cap);
/* Number of visible CUDA devices (0 on a machine without a GPU); never fails. */
int pach_device_count(void);

pach_status pach_scene_create(const pach_scene_desc *desc, pach_scene **out);
/* n scenes at once (a batch's rooms): the host builds (BVH, materials) run on `threads` host threads
 * (0 = all cores); the scenes belong to the calling thread's device.  Each scene's own device copy is
 * made on its first single-room use (pach_trace_begin, pach_trace_specular_paths, pach_direct_sound),
 * since a batch run uploads the concatenation of its rooms instead; pach_trace_run_noalloc, which
 * allocates nothing, needs a scene from pach_scene_create.  On failure no scene is returned. */
pach_status pach_scenes_create(const pach_scene_desc *descs, int32_t n, pach_scene **out, int32_t threads);
void pach_scene_destroy(pach_scene *scene);
/* Scene facts the SplitRayTracer ctor derives (Scene.SurfaceArea, Sound_speed, Rho_C, Attenuation). */
pach_status pach_scene_info(const pach_scene *scene, int32_t *n_polys, int32_t *n_triangles,
                            double *sound_speed, double *rho_c, double air_atten_db_per_m[PACH_BANDS],
                            double *poly_area /* [n_polys] or NULL */);

pach_status pach_trace_begin(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                             const pach_receiver_desc *receivers, int32_t n_receivers,
                             const pach_trace_params *params, pach_run **out);
/* Batch run: many rooms, each with its own scene, sources, receivers, primaries and cutoff, traced as
 * one wavefront (one persistent device loop) -- no counterpart in the reference, which runs one
 * SplitRayTracer per room.  params gives the shared settings (seed, octave range, histogram rate and
 * length, tuning); its ray_count, cutoff_length_m, prim_dirs, prim_weights and proposal are not used
 * (the emission overrides must be NULL).  Room i's primaries are numbered from ray_begin + the rays of
 * rooms 0..i-1, so room i traces exactly as pach_trace_begin would with that ray_begin.  The run's
 * receivers (histogram rows) are the rooms' receivers in room order; scaled histograms divide each
 * room by its own primaries. */
pach_status pach_batch_begin(const pach_room_desc *rooms, int32_t n_rooms, const pach_trace_params *params,
                             pach_run **out);

/* Direct sound of point sources (Direct_Sound.Check_Validity and the unobstructed-path energy,
 * Pachyderm_Acoustic_Universal/Classes_Direct.cs:654-685, 772-823; screen diffraction is not
 * modelled): one visibility ray per (receiver, source) pair on the GPU.  Outputs, row-major by
 * receiver then source: valid (1 = the receiver sees the source directly or through transmissive
 * polygons), distance (m) and energy [..][8] = P 10^(-0.1 m L) prod(tau) / (4 pi L^2) -- the value the
 * reference adds to Io at floor((L / c - Time_Pt) fs).  distance and energy may be NULL. */
pach_status pach_direct_sound(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                              const pach_receiver_desc *receivers, int32_t n_receivers, int32_t *valid,
                              double *distance, double *energy);

/* Autotuner (no counterpart in the reference): times sample runs of the rooms (sample_rays primaries
 * shared among them in proportion to their ray counts) over candidate packet sizes and block shapes,
 * and returns the fastest.  Results are cached in a text file (cache_path, or $PACH_TUNE_CACHE, or
 * ~/.cache/pach_gb300_tune.txt) keyed by device and a coarse workload signature; force = 1 re-tunes.
 * Copy the four knobs into pach_trace_params to use them. */
typedef struct {
    int32_t wave_kilo_items;
    int32_t block_threads;
    int32_t blocks_per_sm;
    int32_t traversal;
    double segments_per_s;         /* the chosen configuration's measured sample throughput */
    double tune_seconds;           /* wall time spent timing (0 when taken from the cache) */
    int32_t trials;                /* configurations timed */
    int32_t from_cache;
} pach_tune_result;
pach_status pach_autotune(const pach_room_desc *rooms, int32_t n_rooms, const pach_trace_params *params,
                          int64_t sample_rays, const char *cache_path, int32_t force, pach_tune_result *out);
pach_status pach_trace_poll(pach_run *run, pach_progress *progress);
pach_status pach_trace_cancel(pach_run *run);
/* Blocks until the run stops or timeout_ms passes (timeout_ms < 0: no limit). */
pach_status pach_trace_wait(pach_run *run, int64_t timeout_ms);
/* Histograms, layouts energy/pressure [R][8][T], dir_pos/dir_neg [R][3][8][T] (+x,+y,+z arrival
 * components), analysis [R][3][8][T] (0 specular, 1 diffuse, 2 specular-after-scatter).
 * scaled = 0: raw sums; 1: Combine_ThreadLocal_Results scaling (energy, dir and analysis / N,
 * pressure / sqrt(N), then x n_sources, pressure x sqrt(n_sources)).  Any pointer may be NULL.
 * cap_bins = capacity of each of energy/pressure in doubles (R*8*T). */
pach_status pach_trace_get_histograms(pach_run *run, int32_t scaled, double *energy, double *pressure,
                                      double *dir_pos, double *dir_neg, double *analysis, size_t cap_bins);
pach_status pach_trace_get_stats(pach_run *run, pach_stats *stats);
/* Map histograms of a run with mapping receivers, energy/pressure [M][8][T] (T = 1 with time_1pt),
 * time 0 = each receiver's direct arrival.  scaled = 1: Histogram.Scale (energy and pressure / N,
 * Classes_Receivers.cs:1211-1218), then x n_sources (Combine_ThreadLocal_Results, TaskAll:768-774).
 * direct_time [M] seconds, sizes [2] = (M, T).  Any pointer may be NULL; cap_bins = capacity of
 * energy and pressure in doubles. */
pach_status pach_trace_get_map(pach_run *run, int32_t scaled, double *energy, double *pressure, double *direct_time,
                               int32_t *sizes, size_t cap_bins);
/* Arrival-direction histograms of a directional map, dir_pos / dir_neg [M][3][8][T] (+x, +y, +z
 * components; Directional_Histogram.Add and Scale, Classes_Receivers.cs:1774-1825: the pressure of a
 * directional map is scaled by 1 / sqrt(N) where a plain map's is scaled by 1 / N).  cap_bins = capacity
 * of each in doubles. */
pach_status pach_trace_get_map_directions(pach_run *run, int32_t scaled, double *dir_pos, double *dir_neg,
                                          size_t cap_bins);
/* Room-acoustic parameters of every map receiver and band, computed on the device from the map
 * histograms (Get_RT_Map, Get_EDT_Map, Get_Clarity_Map, Get_Definition_Map without coherent
 * superposition, Pach_Map_Receiver.cs:925-1270: AcousticalMath.T_X / EarlyDecayTime of the Schroeder
 * integral, Clarity / Definition with the start at bin 0).  Outputs [M][8] (NaN where the decay never
 * reaches the fit limits, as T_X); any may be NULL.  energy_sum = the band's total scaled energy. */
pach_status pach_map_parameters(pach_run *run, int32_t decay_depth, int32_t clarity_ms, double *t_x, double *edt,
                                double *clarity, double *definition, double *energy_sum);
/* The same parameters for n caller curves etc [n][T] at sample_rate Hz (host arrays; the work runs on
 * the current device): T_X / EDT / Clarity (clarity_s seconds) / Definition (50 ms), start time 0. */
pach_status pach_etc_parameters(const double *etc, int32_t n, int32_t T, int32_t sample_rate, int32_t decay_depth,
                                double clarity_s, double *t_x, double *edt, double *clarity, double *definition,
                                double *energy_sum);
void pach_run_destroy(pach_run *run);

/* Synchronous convenience: begin + wait + histograms + stats. */
pach_status pach_trace_run(pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                           const pach_receiver_desc *receivers, int32_t n_receivers,
                           const pach_trace_params *params, int32_t scaled, double *energy, double *pressure,
                           double *dir_pos, double *dir_neg, double *analysis, size_t cap_bins, pach_stats *stats);

/* No counterpart in the reference.  The tracer for callers that must not allocate device memory at
 * trace time -- a host tracing from an audio or plug-in processing callback, or code whose device
 * memory belongs to another framework's allocator: it creates the scene at set-up, then calls this
 * per run with its own device buffers (energy/pressure R*8*T doubles, dir_pos/dir_neg/analysis
 * R*24*T doubles; all five required; cleared by the call).  Its working memory is a fixed ~4.7 MB
 * device array inside the library, resident on every GPU that loads the library until the process
 * exits.  Limits: 16 sources, 256 receivers, 65536 octave rays in flight (a scene whose phase-A bound
 * or split trees need more is rejected with PACH_ERR_INVALID_ARGUMENT or PACH_ERR_BOUNDS), no
 * emission overrides; otherwise it rejects what pach_trace_begin rejects, with the same messages.
 * The scene's device must be current.
 * Set-up: the first call on a device looks up the array's device address (cudaGetSymbolAddress) and
 * may load the library's device code, which allocates device memory once -- make that first call at
 * set-up, before any stream capture, not from the thread that must not allocate.  Later calls
 * allocate nothing.  The address stays cached for the process: after a cudaDeviceReset of that device
 * (which also invalidates its scene handles) this entry point must not be called again.
 * The call is synchronous: it runs on `stream` (a cudaStream_t, NULL = default stream), synchronising
 * it every 32 loop iterations, and returns when the run is done.  Its time grows with ray_count; it
 * returns PACH_ERR_GAVE_UP if the device loop stops making progress for 2048 iterations.  Every call
 * shares the one array, so calls that overlap on the GPU (other threads or streams) race. */
pach_status pach_trace_run_noalloc(const pach_scene *scene, const pach_source_desc *sources, int32_t n_sources,
                                   const pach_receiver_desc *receivers, int32_t n_receivers,
                                   const pach_trace_params *params, void *stream, double *d_energy,
                                   double *d_pressure, double *d_dir_pos, double *d_dir_neg, double *d_analysis,
                                   pach_stats *stats);

/* The convergence checks of convergence mode (TaskAll:783-1107) replayed over a caller's per-revolution
 * histograms, on the host: per_rev [revs][4][T] holds each revolution's raw contribution to one receiver's
 * band-h_oct energy histogram and its three Reflection_Analysis_Data histograms (0 specular, 1 diffuse,
 * 2 specular-after-scatter).  mode 0 = SpecMin_Convergence_Check, 1 = Minimum_Convergence_Check
 * (distance_m / sound_speed = the direct arrival that starts its windows).  *stop_rev = the first
 * revolution (1-based) after which Check() answered true, 0 if none did; *nmin_out = SpecMin's last
 * minimum ray count (may be NULL). */
pach_status pach_convergence_replay(const double *per_rev, int32_t revs, int32_t T, int32_t sample_rate, int32_t mode,
                                    double distance_m, double sound_speed, int32_t *stop_rev, int64_t *nmin_out);

/* Pure-specular paths (oracle (a)): per bounce the hit polygon (-1 = miss), leg length and hit
 * point, traced by the same device traversal as the tracer. */
pach_status pach_trace_specular_paths(pach_scene *scene, int32_t n, const double *origins, const double *dirs,
                                      int32_t max_bounces, int32_t *poly_out, double *t_out, double *pts_out);

/* Builds the scene's BVH on the host and walks it for each ray (FP32 boxes as on the device, FP64
 * triangle tests, t > 1e-10): checks the acceleration structure the kernels use without a GPU.
 * poly_out = -1 on a miss. */
pach_status pach_scene_shoot_host(const pach_scene_desc *desc, int32_t n, const double *origins, const double *dirs,
                                  int32_t *poly_out, double *t_out);

/* Receiver filters (auralisation impulse responses), computed on the GPU in FP64.
 * pach_etc_to_filter: Pach_SP.ETCToFilter (Pach_SP.cs:1584-1680) of n band-pressure envelope sets
 *   prms [n][8][T] at sample_rate Hz: out [n][T + 16383].  Each band's |P| 10^((120 - swl[b]) / 20) is
 *   convolved with a 16384-sample band-limited sinc carrier, plus a 16 kHz band from the 8 kHz
 *   envelope; swl NULL = 120 dB in every band.
 * pach_receiver_filters: Directional_Histogram.Create_Filter(SWL, Rho_C) (Classes_Receivers.cs:1910-1937)
 *   of R receivers' scaled histograms (the pach_trace_get_histograms layouts): out [R][7][T + 12287],
 *   filter 0 from the pressures, 2d+1 / 2d+2 (d = x, y, z) from P Dir_Rec_Neg[d] / E and
 *   P Dir_Rec_Pos[d] / E (0 where E = 0), each cut by 4096 samples as the reference cuts them.  With
 *   dir_pos or dir_neg NULL: Histogram.Create_Filter (1186-1197), out [R][1][T + 12287] (energy unused).
 *   Host arrays; the calling thread's current device computes.
 * pach_trace_get_filters: the same from a finished run's device histograms, scaled as
 *   pach_trace_get_histograms(scaled = 1) scales them, without copying them to the host; directional
 *   = 0 gives filter 0 only.
 * pach_filters_device: device-pointer form, asynchronous on stream (a cudaStream_t; NULL = the legacy
 *   default stream): kinds 1 or 7, cut 0 (ETCToFilter) or 4096 (Create_Filter), d_scale [R] multiplies
 *   each receiver's envelopes (NULL: 1), d_out [R][kinds][T + 16383 - cut]; d_workspace 256-byte
 *   aligned, of at least pach_filters_workspace_bytes(R * kinds, T) bytes (smaller workspaces of at
 *   least one filter's share work in more passes).  T + 16383 <= 2^20. */
pach_status pach_etc_to_filter(const double *prms, int32_t n, int32_t T, const double *swl, int32_t sample_rate,
                               double *out, size_t cap);
pach_status pach_receiver_filters(const double *energy, const double *pressure, const double *dir_pos,
                                  const double *dir_neg, int32_t R, int32_t T, int32_t sample_rate, const double *swl,
                                  double *out, size_t cap);
pach_status pach_trace_get_filters(pach_run *run, int32_t directional, const double *swl, double *out, size_t cap);
size_t pach_filters_workspace_bytes(int32_t n_filters, int32_t T);
pach_status pach_filters_device(const double *d_energy, const double *d_pressure, const double *d_dir_pos,
                                const double *d_dir_neg, const double *d_scale, int32_t R, int32_t T, int32_t kinds,
                                int32_t sample_rate, const double *swl, int32_t cut, double *d_out,
                                void *d_workspace, size_t workspace_bytes, void *stream);

/* Emission directions of primaries [ray_begin, ray_begin+n) as the tracer draws them. */
pach_status pach_emit_directions(uint64_t seed, int64_t ray_begin, int32_t n, int32_t n_sources,
                                 int32_t kind, double *dirs_out);

/* Air: attenuation (dB/m at the 8 octave centres), sound speed (m/s), density (kg/m^3). */
pach_status pach_medium_properties(double temp_c, double rel_humidity, double pressure_hpa, int32_t air_choice,
                                   int32_t edge_correction, double atten_db_per_m[PACH_BANDS],
                                   double *sound_speed, double *rho);
/* The same air model at the reference's third-octave centres (Calculate_Attenuation with Third_Octave,
 * Classes_Medium_Props.cs:51-89, 290): 23 values (its table skips 2500 Hz); centres_hz may be NULL.
 * The reference computes them (Atten_Coef_3rd) but its tracer does not use them: the split ray
 * tracer works in the 8 octave bands. */
pach_status pach_medium_attenuation_third_octave(double temp_c, double rel_humidity, double pressure_hpa,
                                                 int32_t air_choice, int32_t edge_correction, double atten[23],
                                                 double centres_hz[23]);

/* AcousticalMath (Classes_Math.cs). */
pach_status pach_math_schroeder(const double *etc, int32_t n, double *out);              /* 282-299 */
double pach_math_t_x(const double *schroeder, int32_t n, int32_t decay_depth, int32_t sample_f); /* 511-526 */
double pach_math_edt(const double *schroeder, int32_t n, int32_t sample_f);              /* 534-549 */
double pach_math_clarity(const double *etc, int32_t n, double sample_f, double seconds, double start_time,
                         int32_t pressure);                                               /* 559-586 */
double pach_math_definition(const double *etc, int32_t n, double sample_f, double seconds, double start_time,
                            int32_t pressure);                                            /* 934-962 */
double pach_math_center_time(const double *etc, int32_t n, int32_t sample_f, double direct_time,
                             int32_t pressure);                                           /* 971-986 */
double pach_math_strength(const double *etc, int32_t n, double swl, int32_t pressure);   /* 993-1005 */
double pach_math_sound_speed(double temp_c);                                               /* 272-275 */

#ifdef __cplusplus
}
#endif
#endif /* PACH_GPU_H */
