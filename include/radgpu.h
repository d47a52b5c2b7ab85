/*
 * radgpu -- GB300 (sm_103a) wavefront path tracer behind a C ABI.
 *
 * Drop-in replacement for the RadiantiumPlusPlus offline hot path: the
 * `path` and `vol_path` renderers (module/rad.offline/src/renderer/path.cpp,
 * vol_path.cpp), their sample-renderer driver (sample_renderer.cpp) and the
 * Embree accelerator (src/accel/embree.cpp); also the `ao`, `particle_tracer`
 * and `bdpt` renderers (ao.cpp, particle_tracer.cpp, bdpt.cpp). Scenes are the reference's JSON
 * format with the same factory names. Plain pointers and sizes only: no C++
 * or torch types cross this boundary, and no exception escapes it.
 *
 * Every function returns an int status: RAD_OK (0) or one of RAD_ERR_*; the
 * message of the last failure on the calling thread is available from
 * rad_last_error(). Device faults are reported as status words, never traps.
 */
#ifndef RADGPU_H_
#define RADGPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RAD_API __attribute__((visibility("default")))
#else
#define RAD_API
#endif

/* Status codes. RAD_ERR_UNKNOWN_FACTORY mirrors the reference's
 * RadArgumentException("cannot find factory") (rad.core/src/factory.cpp:13-19). */
#define RAD_OK 0
#define RAD_ERR_INVALID_ARG 1
#define RAD_ERR_JSON 2
#define RAD_ERR_UNKNOWN_FACTORY 3
#define RAD_ERR_IO 4
#define RAD_ERR_CUDA 5
#define RAD_ERR_OUT_OF_MEMORY 6
#define RAD_ERR_ADMISSION 7 /* job footprint exceeds the device budget */
#define RAD_ERR_TIMEOUT 8
#define RAD_ERR_CANCELLED 9
#define RAD_ERR_NOT_READY 10
#define RAD_ERR_NO_DEVICE 11
#define RAD_ERR_DEVICE_CHECK 12 /* a device-side bounds/iteration check fired */
#define RAD_ERR_UNSUPPORTED 13

typedef struct rad_scene rad_scene; /* resident scene: BVH8 + materials + lights + media */
typedef struct rad_job rad_job;     /* one render: film, sample counters, queues */

/* Scene summary (camera, sampler and renderer settings from the JSON). */
typedef struct rad_scene_info {
  int32_t width, height;
  int32_t spp;          /* sampler.sample_count (sampler.cpp:6) */
  uint32_t seed;        /* sampler.seed */
  int32_t max_depth;    /* renderer.max_depth, -1 = unbounded */
  int32_t rr_depth;     /* renderer.rr_depth */
  int32_t is_vol_path;  /* 1 for "vol_path", 0 for "path" */
  int32_t n_shapes, n_lights, n_media, n_materials;
  uint64_t n_prims;     /* triangles + analytic primitives */
  uint64_t n_bvh_nodes; /* 8-wide nodes */
  uint64_t device_bytes;
} rad_scene_info;

/* One render request. spp = 0 takes the scene's sample_count; seed = UINT32_MAX
 * takes the scene's sampler seed. first_sample lets a job continue an earlier
 * one with disjoint sample indices (resumable accumulation). For the
 * particle_tracer renderer a sample is one light path over the whole film
 * (particle_tracer.cpp:52-83), so spp counts light paths. A bdpt sample is one
 * camera subpath and one light subpath (bdpt.cpp:261-305). */
typedef struct rad_job_desc {
  uint32_t spp;
  uint32_t seed;
  uint32_t first_sample;
  uint32_t flags; /* RAD_JOB_* */
} rad_job_desc;

#define RAD_JOB_PROFILE_KERNELS 1u /* time every kernel launch with CUDA events */
#define RAD_JOB_SYNC 2u            /* render on the calling thread, return when done */
#define RAD_JOB_COUNT_TRAVERSAL 4u /* count BVH8 node visits / primitive tests (slower) */
#define RAD_JOB_VOL_BRICKS 16u     /* `vol_path`: free flights against 16^3-brick majorants of grid media
                                      instead of the global majorant (fewer null collisions); implies
                                      RAD_JOB_VOL_REAL_DEPTH */
#define RAD_JOB_VOL_FP16 32u       /* `vol_path`: read the density grid's fp16 copy */
#define RAD_JOB_VOL_REAL_DEPTH 64u /* `vol_path`: null collisions count neither toward max_depth nor for
                                      Russian roulette. The reference counts them (vol_path.cpp:40-52
                                      run per loop iteration), so its truncation depends on the majorant */
#define RAD_JOB_VOL_PERSISTENT 128u /* `vol_path`: one persistent kernel instead of the per-event wavefront
                                       (same radiance bit for bit; no wavefront state memory) */
#define RAD_JOB_GUIDE 8u           /* `path` only: sample directions with the scene's learned guide
                                      (one-sample MIS with the BSDF) and train it during the
                                      job's first train_fraction of samples; no reference counterpart */

/* Counters of one job. Rays = primary + extension + shadow rays traced. */
typedef struct rad_stats {
  uint64_t samples;          /* pixel samples finished */
  uint64_t invalid_samples;  /* NaN/Inf/negative samples dropped (sample_renderer.cpp:101-105) */
  uint64_t rays_closest;     /* primary + extension rays */
  uint64_t rays_shadow;
  uint64_t kernel_launches;  /* kernels this library launched for the job */
  double gpu_ms;             /* device time of the job's waves (CUDA events) */
  double wall_ms;            /* host time from start of execution to completion */
  double queue_ms;           /* host time from submit to start of execution */
  /* per-kernel device time when RAD_JOB_PROFILE_KERNELS is set */
  double ms_generate, ms_extend, ms_shade, ms_shadow, ms_accumulate, ms_volpath;
  uint64_t n_extend, n_shade, n_shadow;
  /* with RAD_JOB_COUNT_TRAVERSAL: node visits and primitive tests */
  uint64_t trav_nodes_closest, trav_prims_closest, trav_nodes_shadow, trav_prims_shadow;
  /* with RAD_JOB_GUIDE: training records, Adam steps, and (with RAD_JOB_PROFILE_KERNELS)
   * device time of the guide inference and training stages */
  uint64_t guide_records, guide_train_steps;
  double ms_guide_infer, ms_guide_train;
  /* waves of this job that held paths of other jobs too (mixed waves: plain
   * `path` jobs running together share every launch of a wave; the rays of such
   * a wave are apportioned to its jobs by their shares of its paths) */
  uint64_t mixed_waves;
} rad_stats;

/* ---- library ------------------------------------------------------------ */
/* config_json may be NULL. Keys: "device" (int), "budget_bytes" (admission
 * budget for resident scenes + films, default 150e9), "max_paths" (paths in
 * flight per wave, default 2^21; larger waves raise a lone job's throughput),
 * "bdpt_scratch_bytes" (device bytes a `bdpt` wave's subpath vertices and
 * visibility rays may take, default 2^32; it sets the bdpt wave size), "mix_jobs" (default 1: plain `path` jobs running together
 * share the launches of each wave), "share_exponent" (default 0: a mixed wave
 * gives its jobs path slots in proportion to (remaining samples)^exponent -- 0
 * equal shares, 1 in proportion to the work left), "deadline_ns_per_sample"
 * (default 0 = off; > 0: earliest deadline first, a job's deadline being its
 * submit time + its samples x this allowance, and mixed waves fill their path
 * slots in deadline order), "slowdown_ns_per_sample" (default 0 = off; > 0:
 * highest slowdown first, a job's slowdown being its age over its samples x
 * this + 20 ms, re-evaluated every wave). Idempotent: on a library already
 * initialised only "budget_bytes", "mix_jobs", "share_exponent",
 * "deadline_ns_per_sample" and "slowdown_ns_per_sample" are applied (deadlines
 * of jobs already submitted are kept). */
RAD_API int rad_init(const char* config_json);
RAD_API int rad_shutdown(void);
/* Copies the calling thread's last error message (NUL-terminated). */
RAD_API int rad_last_error(char* buf, size_t size);
RAD_API int rad_version(int32_t* major, int32_t* minor);
/* No counterpart in the reference. Device bytes counted against the admission
 * budget (resident scenes, job films including films parked with a scene for
 * its next job, path-state buffers; the `vol_path` wavefront's per-path states
 * and queues, about 400 B per max_paths slot, from the first `vol_path` wave
 * on) and the budget itself. */
RAD_API int rad_device_usage(uint64_t* used_bytes, uint64_t* budget_bytes);

/* ---- scenes (BuildContext::SetFromJson + Build, build_context.cpp:47-321) -- */
RAD_API int rad_scene_load_json(const char* json_text, const char* base_dir, rad_scene** out);
RAD_API int rad_scene_load_file(const char* path, rad_scene** out);
RAD_API int rad_scene_destroy(rad_scene* scene);
RAD_API int rad_scene_info_get(const rad_scene* scene, rad_scene_info* info);
/* Device bytes the scene holds (BVH + primitives + materials + media). */
RAD_API int rad_scene_footprint(const rad_scene* scene, uint64_t* bytes);

/* ---- jobs (Renderer::Start/Wait/Stop/..., renderer.h:19-48) --------------- */
/* Non-blocking unless RAD_JOB_SYNC: the job joins the serving loop, which
 * admits it once its film fits the device budget and interleaves its waves
 * with the other running jobs. */
RAD_API int rad_job_submit(rad_scene* scene, const rad_job_desc* desc, rad_job** out);
/* timeout_ms < 0 waits forever; returns RAD_ERR_TIMEOUT if not done in time. */
RAD_API int rad_job_wait(rad_job* job, int64_t timeout_ms);
RAD_API int rad_job_cancel(rad_job* job);
/* Thread-safe progress in pixel samples: done, total. */
RAD_API int rad_job_progress(rad_job* job, uint64_t* done, uint64_t* total);
/* Film (sum / spp, sample_renderer.cpp:109-114), row-major RGB fp32, width x height. */
RAD_API int rad_job_film(rad_job* job, float* rgb, int32_t width, int32_t height);
RAD_API int rad_job_stats(rad_job* job, rad_stats* stats);
RAD_API int rad_job_destroy(rad_job* job);

/* ---- parity entry points ------------------------------------------------- */
/* Accel::RayIntersectPreliminary / RayIntersect (accel.h:10-30).
 * rays: n x 8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax), host memory.
 * hits: n x 5 words: closest -> (t, u, v, prim id, front) with prim id =
 * 0xffffffff on a miss (t, u, v floats; prim, front uint32); any -> word 3 is
 * 1 when occluded. Prim id = shape prefix offset + primitive index in shape. */
RAD_API int rad_trace_batch(rad_scene* scene, const float* rays, int64_t n, float* hits, int32_t any_hit);
/* Same on device pointers, on the library's stream, asynchronous. */
RAD_API int rad_trace_batch_device(rad_scene* scene, const float* d_rays, int64_t n, float* d_hits, int32_t any_hit);
/* Bsdf::Eval + Bsdf::Pdf (bsdf.h:103-142) for one BSDF given as reference JSON,
 * e.g. {"type":"rough_metal","alpha":0.2}. wi, wo: n x 3 local directions;
 * f: n x 3 (cosine-weighted); pdf: n. Host memory. */
RAD_API int rad_bsdf_eval_batch(const char* bsdf_json, const float* wi, const float* wo, int64_t n, float* f,
                                float* pdf);
/* Bsdf::Sample. u: n x 3 (lobe, dir.x, dir.y). Outputs as the reference's
 * BsdfSampleResult: wo n x 3, pdf n, f n x 3, eta n, type n (BsdfType bits). */
RAD_API int rad_bsdf_sample_batch(const char* bsdf_json, const float* wi, const float* u, int64_t n, float* wo,
                                  float* pdf, float* f, float* eta, uint32_t* type);
/* Perspective::SampleRay (perspective.cpp:73-82) for pixel samples, jitter from
 * each sample's own stream. pixels: n (x + y * width); out: n x 8 rays. */
RAD_API int rad_camera_rays(rad_scene* scene, const uint32_t* pixels, int64_t n, uint32_t sample, uint32_t seed,
                            float* rays);
/* Texture<T>::Eval (texture.h:57-62) of the scene's texture number `texture`
 * (textures are numbered in the order the scene file creates them: BSDF
 * parameters in each factory's reading order, a chessboard before its two
 * children). uv: n x 2; duv: n x 4 (du/dx, dv/dx, du/dy, dv/dy); out: n x 3
 * (mono textures fill the first column). Host memory. */
RAD_API int rad_scene_texture_eval(rad_scene* scene, uint32_t texture, const float* uv, const float* duv, int64_t n,
                                   float* out);
/* Radiance of individual pixel samples (Li), n x 3, through the same kernels
 * as a job. For bdpt: the camera-side sum (connections with t >= 2 camera
 * vertices); its t = 1 connections land on other pixels and are left out.
 * RAD_ERR_UNSUPPORTED for particle_tracer. */
RAD_API int rad_render_samples(rad_scene* scene, const uint32_t* pixels, const uint32_t* samples, int64_t n,
                               uint32_t seed, float* radiance);

/* ---- allocation-free variant --------------------------------------------- */
/* No counterpart in the reference. Same result as rad_render_samples, for
 * callers that cannot call cudaMalloc (a host whose device memory is all
 * handed to its own pool, or a frame loop that must not let allocations
 * synchronise the device): d_pixels, d_samples (n each) and d_radiance (n x 3)
 * are device pointers the caller owns, and the path state lives in a fixed
 * file-scope device array, so this call allocates nothing. n may be at most
 * 16384 (RAD_ERR_INVALID_ARG beyond). The pixel indices are in device memory,
 * so the host cannot check them: one beyond the film is reported as
 * RAD_ERR_DEVICE_CHECK after the call (rad_render_samples, which reads them
 * on the host, answers RAD_ERR_INVALID_ARG). Work runs on `stream` (a cudaStream_t,
 * NULL = default stream) and the call returns when it has finished. The first
 * call on a device looks up the array's address; make it before any stream
 * capture. Every call shares the one array: calls that overlap on the GPU race.
 * RAD_ERR_UNSUPPORTED for particle_tracer (no per-pixel samples) and bdpt (its
 * subpaths live in scratch the library allocates). */
RAD_API int rad_render_samples_noalloc(rad_scene* scene, const uint32_t* d_pixels, const uint32_t* d_samples,
                                       int64_t n, uint32_t seed, float* d_radiance, void* stream);

/* ---- learned path guiding ------------------------------------------------ */
/* No counterpart in the reference (its integrators sample the BSDF only). A
 * scene may own one guide network: a 16-level hash grid over the shading
 * position (2 features per level, 2^log2_table entries each) plus the shading
 * normal and outgoing direction, into a 3 x 64 ReLU MLP (fp16 weights, fp32
 * accumulation) whose 41 outputs give an 8-lobe von Mises-Fisher mixture over
 * world directions and the probability c <= c_max of sampling it instead of
 * the BSDF. Jobs submitted with RAD_JOB_GUIDE sample p = c q + (1 - c) p_bsdf
 * (unbiased for any network state) and train the network online with Adam on
 * their own paths during their first train_fraction of samples. */
typedef struct rad_guide_info_t {
  uint64_t n_params;   /* table + MLP weights */
  uint64_t n_table;    /* levels x 2^log2_table x 2 */
  uint32_t log2_table, levels;
  uint32_t level_res[16];
  float lo[3], hi[3];  /* world box mapped to the unit cube */
  uint64_t adam_steps;
  uint64_t device_bytes;
} rad_guide_info_t;

/* Creates (or re-creates, seeded) the scene's guide. config_json may be NULL;
 * keys: log2_table (19), min_res (16), max_res (512), lr (0.01, hash table),
 * lr_mlp (0.001), train_fraction (0.25), train_path_shift (4: 1 in 16 paths
 * records training vertices), train_depth (8), steps_per_wave (8),
 * record_capacity (2^20), weight_clamp (32), log_kappa_max (5), c_max (0.6),
 * seed (5), lazy_table (1: an Adam step leaves hash-table entries without a
 * gradient in its batch untouched; 0: every parameter takes every step). A
 * checkpoint carries the network, not these settings. Fails while jobs of the
 * scene are live. */
RAD_API int rad_guide_enable(rad_scene* scene, const char* config_json);
RAD_API int rad_guide_info(rad_scene* scene, rad_guide_info_t* info);
/* Serialises parameters and Adam moments into buf (host); *needed gets the
 * size. buf = NULL only queries the size. */
RAD_API int rad_guide_checkpoint(rad_scene* scene, void* buf, size_t size, size_t* needed);
/* Replaces the scene's guide with a checkpoint's (RAD_ERR_INVALID_ARG if malformed). */
RAD_API int rad_guide_load(rad_scene* scene, const void* buf, size_t size);
/* Network on queries (n x 9: position, shading normal, outgoing direction;
 * world space). raw (n x 48, optional): outputs; mix (n x 44, optional):
 * 8 x (mu xyz, kappa), 8 lobe weights, c, 3 zeros. Creates a default guide if
 * the scene has none. Host memory. */
RAD_API int rad_guide_forward(rad_scene* scene, const float* queries, int64_t n, float* raw, float* mix);
/* Mixture pdf of packed mixtures (n x 44 as above): at dirs (n x 3) when dirs
 * is given, else of directions sampled from u (n x 3: lobe, two direction
 * numbers) returned in out_dirs. Exactly one of dirs / u. Host memory. */
RAD_API int rad_guide_mix_eval(const float* mix, const float* dirs, const float* u, int64_t n, float* pdf,
                               float* out_dirs);
/* Gradient of sum_i -w_i log p_i(wi_i) over records (n x 16: position, p_bsdf |
 * normal, - | wo, - | wi, w) with respect to every parameter (grad: n_params,
 * table first, summed over records); loss gets the summed loss. The same
 * kernels as training. Host memory. */
RAD_API int rad_guide_grad(rad_scene* scene, const float* records, int64_t n, float* grad, float* loss);

/* ---- autotuner ------------------------------------------------------------ */
/* No counterpart in the reference (its TBB tiles need no tuning). Picks the
 * launch parameters of the `path` traversal kernels for a scene by timing full
 * 1-spp waves, one axis at a time from the defaults (coordinate descent): the
 * fraction of a warp's busy lanes that must hold pending leaves before it tests
 * leaves (leaf_frac8 / 8), the warp refill threshold of the persistent
 * closest-hit and shadow kernels (lanes still tracing before idle lanes take new
 * rays), the number of blocks per SM of their grids, and the block size of the
 * shade-class kernels. The winner is kept in the scene and used by later jobs,
 * mixed waves and rad_render_samples; results do not depend on it. config_json
 * may be NULL; keys: leaf_frac8 (list, default [2,3,4,5,6]), refill_busy (list,
 * default [16,20,24,28,32]), blocks_per_sm (list, default [4,6,8]),
 * shade_block (list of 64 / 128 / 256, default all three), reps (timed waves
 * per candidate, 2).
 * `vol_path` scenes: the axes are those of the per-event wavefront's part
 * kernels -- refill_busy (a warp tops up its lanes once fewer than this many
 * still run a path; default [8,12,16,20,24,28,32]), blocks_per_sm (default
 * [2,3,4]; 4 is the kernels' occupancy, larger values run as 4) and vol_chunk
 * (steps of a repeating part -- null collisions, NEE transmittance -- a lane runs
 * per path and launch before the path continues in the next round; default
 * [4,8,16,32,64]); leaf_frac8 and shade_block do not apply. Waves use the
 * reference's estimator on the fp32 grid.
 * RAD_ERR_UNSUPPORTED for `particle_tracer` and `bdpt` scenes. */
typedef struct rad_tune_result {
  int32_t refill_busy, blocks_per_sm; /* chosen */
  int32_t candidates;                 /* configurations timed */
  double best_ms;    /* time of one wave with the chosen parameters */
  double default_ms; /* with the defaults (20, 8, 4, 128, 16), when they were timed */
  int32_t leaf_frac8; /* chosen */
  int32_t shade_block; /* chosen */
  int32_t vol_chunk;   /* chosen (`vol_path`; 16 elsewhere) */
} rad_tune_result;
RAD_API int rad_autotune(rad_scene* scene, const char* config_json, rad_tune_result* out);

#ifdef __cplusplus
}
#endif
#endif /* RADGPU_H_ */
