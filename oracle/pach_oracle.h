/*
 * pach_oracle.h -- CPU FP64 restatement of Pachyderm's stochastic split ray tracer.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The product
 * (libpach_gpu.so) never links, loads or calls it.
 *
 * Parity status: UNPINNED against the reference itself.  The reference is C# (no .NET runtime
 * here), its geometry kernel (Hare.Geometry: Voxel_Grid.Shoot, Topology.intersect,
 * Polygon.GetRandomPoint) is an unvendored, unversioned project reference, and the reference
 * ships no tests, fixtures or golden vectors.  The restatement is instead pinned to analytic
 * known answers (shoebox image-lattice paths, the ISO 9613-1 formula as coded, ideal
 * exponential decays for the room-acoustic parameters, Lambert split expectations).
 *
 * Every function cites the reference file:line it restates; paths are relative to
 * Pachyderm_Acoustic_Universal/.  "TaskAll" is "Classes_Complete_Trace - TaskAll.cs".
 */
#ifndef PACH_ORACLE_H
#define PACH_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scene: polygons over a shared vertex list, 8-band coefficients per polygon, air state.
 * Mirrors Polygon_Scene.Construct (Classes_Scenes.cs:447-630) + Scene ctor (Classes_Scenes.cs:70-105). */
typedef struct {
    int32_t n_vertices;
    const double *vertices;        /* [3*n_vertices] */
    int32_t n_polys;
    const int32_t *poly_offsets;   /* [n_polys+1] into poly_indices */
    const int32_t *poly_indices;
    const double *absorption;      /* [n_polys*8] alpha per octave band 62.5 Hz..8 kHz */
    const double *scattering;      /* [n_polys*8] scattering coefficient s */
    const double *transmission;    /* [n_polys*8] or NULL */
    double temp_c;                 /* degC */
    double rel_humidity;           /* percent */
    double pressure_hpa;           /* hPa (Scene ctor argument; 1013.25 = 101.325 kPa) */
    int32_t air_choice;            /* 0 ISO 9613-1, 1 Evans-Bazley, 2 tables */
    int32_t edge_correction;
} orc_scene_desc;

typedef struct {
    double origin[3];
    double power_db[8];            /* sound power level per octave band, dB re 1e-12 W */
    int32_t kind;                  /* 0 geodesic (GeodesicSource), 1 random (RandomSource), 2 uniform sphere */
    int32_t pad;
} orc_source;

typedef struct {
    double origin[3];
    double radius;
} orc_receiver;

typedef struct {
    uint64_t seed;
    double cutoff_length_m;        /* SplitRayTracer ctor "cutoffTime" (a length): COTime = L / c */
    int32_t oct_lo, oct_hi;        /* octave range, inclusive */
    int32_t is_order;              /* image-source order already covered; -1 = rays record the direct path */
    int32_t sample_rate;           /* histogram rate, Hz */
    double hist_cotime_ms;         /* histogram length in ms (Receiver_Bank COTime_in) */
    int32_t pure_specular;         /* 1: every scattering/transmission coefficient and Lambert threshold forced to 0 */
    int32_t grid_domain;           /* voxel cells per axis (Pach_Properties default 7) */
    int32_t brute_force;           /* 1: nearest hit by testing every polygon (grid cross-check) */
    int32_t max_broadband_bounces; /* 0 = derived bound */
    int64_t max_segments_per_ray;  /* safety cap per octave ray (0 = 1<<22) */
} orc_params;

typedef struct {
    int64_t primaries;
    int64_t segments;              /* shoot calls: broadband + octave, hit or miss */
    int64_t segments_broadband;
    int64_t segments_phase_b;
    int64_t segments_phase_c;
    int64_t octave_rays;           /* octave rays created */
    int64_t end_traces;            /* _rayTotal: octave rays entering End_Trace */
    int64_t detections;
    int64_t capped;                /* rays stopped by a safety cap */
    int64_t cells_visited;         /* voxel cells stepped by the reference traversal (all segments) */
    int64_t tri_tests;             /* polygon tests after mailboxing (all segments) */
    double lost_energy;
    double initial_energy;
    int32_t h_oct;
    int32_t bins;
    double cotime_s;
    double sound_speed;
    double rho_c;
    double air_atten_db_per_m[8];
} orc_stats;

/* Air properties: Uniform_Medium ctor (Classes_Medium_Props.cs:286-299). */
void orc_medium(double temp_c, double hr, double pa_hpa, int air_choice, int edge_correction,
                double atten_db_per_m[8], double *sound_speed, double *rho);

/* Trace primaries [ray_begin, ray_end) with n_threads host threads.  Histograms are RAW sums
 * (not divided by the ray count); layout energy/pressure [R][8][T], dir_pos/dir_neg [R][3][8][T],
 * analysis [R][3][8][T] (0 spec, 1 diffuse, 2 specular-after-scatter).  Returns 0 on success. */
int orc_trace(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
              int32_t n_rec, const orc_receiver *rec, const orc_params *p,
              int64_t ray_begin, int64_t ray_end, int32_t n_threads,
              double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
              orc_stats *stats);

/* As orc_trace, with the emission direction and energy weight of each primary supplied by the
 * caller (prim_dirs [N][3], prim_weights [N], indexed by ray - ray_begin; either may be NULL).
 * This is how an importance-sampled emission (weight 1/q) is checked. */
int orc_trace_ex(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
                 int32_t n_rec, const orc_receiver *rec, const orc_params *p,
                 int64_t ray_begin, int64_t ray_end, int32_t n_threads,
                 const double *prim_dirs, const double *prim_weights,
                 double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
                 orc_stats *stats);

/* Mapping receivers (PachMapReceiver, Pach_Map_Receiver.cs): spheres of diameter `increment` at
 * the given centres, the reference's receiver grid and walks (walk 0) or every crossed cell
 * (walk 1), Map_Receiver detection, 1000 Hz histograms counted from each receiver's direct
 * arrival; time_1pt = Histogram_1Pt. */
typedef struct {
    int32_t n_receivers;
    int32_t time_1pt;
    const double *origins;         /* [3*n_receivers] */
    double increment;
    double cutoff_ms;
    int32_t walk;
    int32_t directional;           /* Directional_Histogram: pressure sqrt(E rho c), +-x/y/z arrival sums */
} orc_map_desc;

/* As orc_trace_ex with mapping receivers as well (map may be NULL): map_energy / map_pressure
 * [M][8][Tm] RAW sums, Tm = (int)(cutoff_ms / 1000 * 1000) or 1; map_direct [M] seconds.  Any
 * output pointer may be NULL. */
int orc_trace_map(const orc_scene_desc *scene, int32_t n_src, const orc_source *src,
                  int32_t n_rec, const orc_receiver *rec, const orc_map_desc *map, const orc_params *p,
                  int64_t ray_begin, int64_t ray_end, int32_t n_threads,
                  const double *prim_dirs, const double *prim_weights,
                  double *energy, double *pressure, double *dir_pos, double *dir_neg, double *analysis,
                  double *map_energy, double *map_pressure, double *map_direct, orc_stats *stats);

/* The direction histograms [M][3][8][Tm] of the last orc_trace_map call on this thread with a
 * directional map (RAW sums); returns 0 when there are none. */
int orc_map_directions(double *dir_pos, double *dir_neg, size_t cap);

/* Pure specular path of each ray: per bounce the hit polygon (-1 = miss, then stop), the leg
 * length and the hit point.  Used for the image-lattice known answers. */
int orc_specular_paths(const orc_scene_desc *scene, int32_t grid_domain, int32_t brute_force,
                       int32_t n, const double *origins, const double *dirs, int32_t max_bounces,
                       int32_t *poly_out, double *t_out, double *pts_out);

/* Nearest hit of one ray (t > 1e-10) -- grid and brute force share this entry. */
int orc_direct(const orc_scene_desc *scene, int32_t grid_domain, int32_t n_src, const orc_source *src,
               int32_t n_rec, const orc_receiver *rec, int32_t *valid, double *distance, double *energy);
int orc_shoot(const orc_scene_desc *scene, int32_t grid_domain, int32_t brute_force,
              const double o[3], const double d[3], int32_t *poly, double *t, double hit[3]);

/* The RNG shared by the oracle and the GPU engine (Philox4x32-10, counter-based). */
void orc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t out[4]);

/* Emission direction of primary `ray` (kind as orc_source.kind). */
void orc_emit_direction(uint64_t seed, int64_t ray, int32_t n_src, int32_t kind, double dir[3]);

/* Room-acoustic parameters (Classes_Math.cs). */
void orc_schroeder(const double *etc, int32_t n, double *out);
double orc_t_x(const double *schroeder, int32_t n, int32_t decay_depth, int32_t sample_f);
double orc_edt(const double *schroeder, int32_t n, int32_t sample_f);
double orc_clarity(const double *etc, int32_t n, double sample_f, double seconds, double start_time, int32_t pressure);
double orc_definition(const double *etc, int32_t n, double sample_f, double seconds, double start_time, int32_t pressure);
double orc_center_time(const double *etc, int32_t n, int32_t sample_f, double direct_time, int32_t pressure);
double orc_strength(const double *etc, int32_t n, double swl, int32_t pressure);

#ifdef __cplusplus
}
#endif
#endif
