/* ard_gb300.h -- C ABI of the GB300 ARD time-step library (libard_gb300.so).
 *
 * The library replaces the per-step loop of pjx3/ARD-simulator,
 * Simulation::Update (ARD-simulator-190113/simulation.cpp:300-318), with
 * hand-written sm_103a CUDA kernels.  The reference's object model stays the
 * host-side description: a scene is the flattened list of partitions
 * (Partition / DctPartition / PmlPartition), boundaries (Boundary), sound
 * sources (SoundSource) and recorders (Recorder), in the reference's own list
 * order, because the order decides which interface wins where interface
 * strips overlap (boundary.cpp:21-173 overwrites; one thread => last wins).
 *
 * All entry points are plain C: integers, floats, pointers and sizes.  Every
 * call returns ARD_OK (0) or an ARD_ERR_* code; ard_last_error() gives the
 * message.  The caller owns host buffers; a context owns its device memory.
 * A context is used from one host thread at a time; contexts are independent.
 * Cells are integers in units of dh; fields are float32, row-major [z][y][x]
 * with x fastest, as in DctVolume (dct_volume.cpp:72) and PmlPartition
 * (pml_partition.cpp:6-15).
 */
#ifndef ARD_GB300_H
#define ARD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ARD_ABI_VERSION 1

/* ---- status codes ---- */
enum {
  ARD_OK = 0,
  ARD_ERR_INVALID = 1,   /* malformed scene or argument */
  ARD_ERR_CUDA = 2,      /* CUDA runtime error (message has the CUDA name) */
  ARD_ERR_OOM = 3,       /* device allocation failed */
  ARD_ERR_STATE = 4,     /* call not valid in the context's current state */
  ARD_ERR_UNSTABLE = 5,  /* non-finite recorder sample or dt over the PML CFL limit */
  ARD_ERR_RANGE = 6,     /* index / time range outside what the context holds */
  ARD_ERR_NOGPU = 7      /* no CUDA device, or the kernels were not built for it */
};

/* Partition kinds: DctPartition / PmlPartition. */
enum { ARD_PART_DCT = 0, ARD_PART_PML = 1 };

/* PmlPartition::PmlType, same order (pml_partition.h:39-46). */
enum {
  ARD_PML_LEFT = 0,
  ARD_PML_RIGHT = 1,
  ARD_PML_TOP = 2,
  ARD_PML_BOTTOM = 3,
  ARD_PML_FRONT = 4,
  ARD_PML_BACK = 5
};

/* Boundary::BoundaryType, same order (boundary.h:30-34). */
enum { ARD_BOUNDARY_X = 0, ARD_BOUNDARY_Y = 1, ARD_BOUNDARY_Z = 2 };

/* One Partition (partition.h:13-74): cell origin and extent. */
typedef struct ard_partition {
  int32_t kind;      /* ARD_PART_DCT or ARD_PART_PML */
  int32_t pml_type;  /* ARD_PML_* for PML partitions, -1 for DCT partitions */
  int32_t x_start, y_start, z_start;
  int32_t width, height, depth;
} ard_partition;

/* One Boundary (boundary.h:9-46): a_ and b_ are indices into the scene's
 * partition list; the ranges are Boundary::x_start_ .. z_end_. */
typedef struct ard_boundary {
  int32_t type;  /* ARD_BOUNDARY_* */
  int32_t a, b;
  int32_t x_start, x_end, y_start, y_end, z_start, z_end;
  float absorption;
} ard_boundary;

/* A sound source or recorder at a global cell.  partition is the air
 * partition it belongs to: for sources the one whose half-open box holds the
 * cell (simulation.cpp:37-48), for recorders the first one that passes
 * Recorder::FindPartition's 5-cell margin test (recorder.cpp:26-38). */
typedef struct ard_point {
  int32_t x, y, z;
  int32_t partition;
} ard_point;

/* A whole scene: the reference's Simulation after its constructor ran.
 * partitions: air partitions first, then PMLs, as Simulation::m_partitions.
 * boundaries: Simulation::m_boundaries order. */
typedef struct ard_scene {
  float dh;             /* Simulation::m_dh (m) */
  float dt;             /* Simulation::m_dt (s) */
  float c0;             /* Simulation::m_c0 (m/s) */
  int32_t pml_layers;   /* Simulation::m_pml_layers */
  float pml_R;          /* PmlPartition::R_ (pml_partition.h:8), 1e-5 */
  float modal_damping;  /* DctPartition::Update's 0.999f (dct_partition.cpp:68) */
  int32_t n_partitions;
  const ard_partition* partitions;
  int32_t n_boundaries;
  const ard_boundary* boundaries;
  int32_t n_sources;
  const ard_point* sources;
  int32_t n_recorders;
  const ard_point* recorders;
} ard_scene;

/* ===================================================================== */
/* Host-side scene construction (no GPU needed).                          */
/* ===================================================================== */

/* Parameters of a scene build; the reference keeps them as static members
 * set in main.cpp:29-45. */
typedef struct ard_scene_params {
  float dh, dt, c0;
  int32_t pml_layers;
  float absorption;     /* Partition::m_absorption, used for PML interfaces */
  float pml_R;          /* 0 selects 1e-5 */
  float modal_damping;  /* 0 selects 0.999 */
} ard_scene_params;

typedef struct ard_scene_buf ard_scene_buf;

/* Builds a scene from air partitions given as cell boxes (6 ints each:
 * x, y, z, width, height, depth), exactly as Simulation::Simulation
 * (simulation.cpp:14-294) does: pairwise Boundary::FindBoundary
 * (boundary.cpp:289-334) with Partition::AddBoundary's free-border marking
 * (partition.cpp:96-143), source attachment, then per air partition the
 * left/right/top/bottom PML runs over z-slice 0 of the free-border maps and
 * the always-present front and back PMLs, each with its interface.
 * Recorders get their partition by Recorder::FindPartition.
 * src_cells / rec_cells hold 3 ints (x, y, z) per point. */
int ard_scene_build(const ard_scene_params* params,
                    int32_t n_air, const int32_t* air_boxes,
                    int32_t n_sources, const int32_t* src_cells,
                    int32_t n_recorders, const int32_t* rec_cells,
                    ard_scene_buf** out);

/* Same, reading the reference's integer-metre text files (README.md:13-37;
 * Partition::ImportPartitions partition.cpp:151-176,
 * SoundSource::ImportSources sound_source.cpp:24-48,
 * Recorder::ImportRecorders recorder.cpp:67-89): each value is divided by dh
 * in float and truncated to int.  recorders_path may be NULL. */
int ard_scene_import(const ard_scene_params* params,
                     const char* partitions_path,
                     const char* sources_path,
                     const char* recorders_path,
                     ard_scene_buf** out);

/* The scene held by a buffer (valid until ard_scene_free). */
const ard_scene* ard_scene_get(const ard_scene_buf* buf);
void ard_scene_free(ard_scene_buf* buf);

/* Message of the last failed scene build on this thread. */
const char* ard_scene_last_error(void);

/* GaussianSource::SampleValue (gaussian_source.cpp:16-20) for t = 0..n-1:
 * 1e9 * exp(-(pi * (2 * (c0*dt/dh) * t / 6 - 2))^2), evaluated in float. */
int ard_gaussian_series(float c0, float dt, float dh, int64_t n, float* out);

/* ===================================================================== */
/* GPU time stepping.                                                     */
/* ===================================================================== */

typedef struct ard_ctx ard_ctx;

enum { ARD_PREC_F32 = 0, ARD_PREC_F64 = 1 };

typedef struct ard_options {
  int32_t precision;     /* ARD_PREC_F32 (product path) or ARD_PREC_F64 (GPU oracle) */
  int64_t max_steps;     /* capacity of source series and recorder history */
  int32_t use_graphs;    /* capture step sequences in CUDA graphs (default 1) */
  int32_t device;        /* CUDA device ordinal */
  int32_t autotune;      /* nonzero: build each candidate layout (modal tile counts,
                            lanes per ky row, fused or GEMM face transforms), time
                            128 steps of each, keep the fastest (default 0) */
  int32_t arithmetic;    /* ARD_ARITH_ACCURATE (default) or ARD_ARITH_REFERENCE */
  int32_t adjoint;       /* nonzero: allocate the adjoint state (needed by ard_adjoint) */
} ard_options;

/* Modal-update arithmetic of the air partitions.
 * ACCURATE: tables 1 - cos(w dt) and 2 (1 - cos(w dt)) / w^2 built in FP64,
 *   update M+ = a ((2M - M-) - 2 (1 - cos) M + psi F); no cancellation near
 *   cos = 1, so FP32 stays within 1e-4 of the FP64 solution.
 * REFERENCE: the reference's own FP32 tables (w and cos(w dt) in float,
 *   dct_partition.cpp:24-36) and update order (dct_partition.cpp:66-68);
 *   reproduces the reference's FP32 rounding, whose error against FP64
 *   reaches ~2e-4 on long runs. */
enum { ARD_ARITH_ACCURATE = 0, ARD_ARITH_REFERENCE = 1 };

/* Creates a context holding n_scenes independent scenes.  n_scenes > 1 is the
 * batched mode: every stage runs as one launch over all scenes' work tables.
 * opt may be NULL (defaults: f32, max_steps 4096, graphs on, device 0). */
int ard_create(const ard_scene* scenes, int32_t n_scenes,
               const ard_options* opt, ard_ctx** out);
int ard_destroy(ard_ctx* ctx);

/* Time series injected by source `source` of scene `scene` (replaces the
 * default all-zero series).  Sample t is written into the force cell at step
 * t, as Partition::ComputeSourceForcingTerms (partition.cpp:187-197) does
 * with SoundSource::SampleValue(t).  n <= max_steps.  scene = source = -1
 * sets every source of every scene at once from series[n_sources_total][n]
 * (sources numbered scene by scene). */
int ard_set_source_series(ard_ctx* ctx, int32_t scene, int32_t source,
                          const float* series, int64_t n);

/* Samples t0 .. t0+n-1 of the series of source `source` of scene `scene`;
 * the other samples stay as they are (the streaming form of
 * ard_set_source_series: a host that produces the source signal block by
 * block uploads each block before the steps that inject it, as
 * SoundSource::SampleValue (sound_source.h:18) is sampled step by step).
 * t0 + n <= max_steps.  scene = source = -1 writes every source of every
 * scene from samples[n_sources_total][n].  Synchronous. */
int ard_set_source_samples(ard_ctx* ctx, int32_t scene, int32_t source, int64_t t0, int64_t n,
                           const float* samples);

/* Initial pressure of air partition `partition` (width*height*depth floats,
 * [z][y][x]).  Sets both modal time levels so that the partition starts at
 * rest with this pressure.  Only before the first step (or after reset). */
int ard_set_initial_pressure(ard_ctx* ctx, int32_t scene, int32_t partition,
                             const float* pressure);

/* Per-face multipliers of the PML damping profile zeta (pml_partition.cpp:
 * 69-86), indexed by ARD_PML_*.  Default all 1. */
int ard_set_pml_scale(ard_ctx* ctx, int32_t scene, const float scale[6]);

/* Zeroes all state and sets the step counter to 0 (series and scales stay). */
int ard_reset(ard_ctx* ctx);

/* Advances every scene by nsteps steps on `stream` (a cudaStream_t; NULL
 * means the context's own stream).  Stream-ordered: returns once the work is
 * queued.  Each step is Simulation::Update's phase A (source forcing, air
 * partition modal update, PML update) then phase B (interface forcing). */
int ard_step(ard_ctx* ctx, int64_t nsteps, void* stream);

/* Waits for all work queued on the context's streams. */
int ard_synchronize(ard_ctx* ctx);

/* Current step counter (number of steps taken since create/reset). */
int ard_time_step(const ard_ctx* ctx, int64_t* out);

/* Recorder samples of scene `scene` for steps t0 .. t0+nt-1, written as
 * out[t][recorder] (n_recorders floats per step; scene = -1: every recorder
 * of every scene, numbered scene by scene).  The sample of step t is
 * the pressure after step t's update, as Recorder::RecordField
 * (recorder.cpp:40-57) takes it after Simulation::Update.  Synchronous. */
int ard_read_recorders(ard_ctx* ctx, int32_t scene, float* out, int64_t t0, int64_t nt);

/* Same samples in double precision (the FP64 context keeps them in double). */
int ard_read_recorders_f64(ard_ctx* ctx, int32_t scene, double* out, int64_t t0, int64_t nt);

/* Current pressure field of partition `partition` of scene `scene`
 * (width*height*depth floats, [z][y][x]).  Synchronous.  For an air
 * partition this runs the full inverse transform of the current modes. */
int ard_read_field(ard_ctx* ctx, int32_t scene, int32_t partition, float* out);

/* Text output in the reference's formats (output/README.md): for scene
 * `scene`, response_<r>.txt per recorder (the recorded pressure of steps
 * 0 .. nt-1, one value per line, as Recorder::RecordField's response stream,
 * recorder.cpp:15-16,55) and source_<s>.txt per source (the injected series,
 * as SoundSource::RecordSource, sound_source.cpp:50-56), in directory `dir`
 * (which must exist).  When the neighbourhoods were recorded from step 0
 * (ard_record_neighbourhoods), also out_<r>.txt per recorder: one line per
 * step with the 1000 values of the 10x10x10 cube, each followed by a space,
 * as Recorder::RecordField's output stream (recorder.cpp:13-14,44-53).
 * Synchronous. */
int ard_write_outputs(ard_ctx* ctx, int32_t scene, const char* dir, int64_t nt);

/* Recorder::RecordField's neighbourhood stream (recorder.cpp:40-57): with
 * enable != 0 every following step also records, for every recorder of every
 * scene, the pressure of the 10x10x10 cube of cells (x+k, y+j, z+i),
 * i, j, k = -5 .. 4, after the step's update, kept on the device for
 * max_steps steps (max_steps * n_recorders * 4000 bytes, allocated here).
 * The cube is contracted from the partition's modes, three extra launches
 * per step inside the step graph.  Every recorder's cube must lie inside its
 * partition (Recorder::FindPartition's margin), else ARD_ERR_INVALID.
 * enable = 0 frees the history.  Synchronous. */
int ard_record_neighbourhoods(ard_ctx* ctx, int32_t enable);

/* Recorded neighbourhoods of steps t0 .. t0+nt-1 of scene `scene` (-1: all
 * scenes), as out[t][recorder][1000] with the cube in the reference's order
 * (z offset slowest, x offset fastest).  Steps before the recording was
 * enabled (or before the last ard_reset) are ARD_ERR_RANGE.  Synchronous. */
int ard_read_neighbourhoods(ard_ctx* ctx, int32_t scene, float* out, int64_t t0, int64_t nt);

/* Size of scene `scene`'s visualization image (Simulation::Simulation's
 * size_x_ / size_y_ / size_z_, simulation.cpp:272-288: the bounding box of
 * all partitions, PMLs included): look_from 0 (xy) gives size_x x size_y,
 * look_from 1 (yz) size_y x size_z (width = row length). */
int ard_slice_size(ard_ctx* ctx, int32_t scene, int32_t look_from, int32_t* width, int32_t* height);

/* Headless form of Simulation::Update's visualization block
 * (simulation.cpp:320-420): the colour map of a pressure slice into the
 * caller's device buffer of width*height RGBA8888 words (ard_slice_size).
 * look_from 0: the xy plane, 1: the yz plane; `coord` is the reference's
 * pixels_z / pixels_x (the first source's z or x).  As the reference does,
 * every partition (air and PML, in list order, later ones overwriting
 * earlier ones) whose extent along the view axis reaches coord (end
 * inclusive) is drawn, and coord is passed to it as a local coordinate;
 * values outside the partition read 0 (PmlPartition::GetIndex's sentinel;
 * the reference's air partitions read outside their array there).  Colour:
 * norm = 0.5 clamp(p v_coef, -1, 1) + 0.5 (v_coef = 10 in the reference),
 * word SDL_MapRGBA(RGBA8888, 255, r, g, b) = 0xFF000000 | r<<16 | g<<8 | b.
 * Pixels no partition covers are left as they are.  pressure_device (may be
 * NULL) receives the drawn pressure values in the same layout.
 * Synchronous. */
int ard_render_slice(ard_ctx* ctx, int32_t scene, int32_t look_from, int32_t coord, float v_coef,
                     uint32_t* pixels_device, float* pressure_device);

/* Room impulse response and reverberation time of matlab/auralization.m
 * (:22-36) and matlab/t60.m, in FP64 on the device over the recorded
 * pressure of recorder `recorder` and the injected series of source
 * `source` of scene `scene`, steps 0 .. nt-1:
 *   rr = response, zeroed from sample `truncate` on (truncate <= 0: kept
 *        whole; auralization.m:25-27 truncates at its Sabine estimate);
 *   rir = the first nt samples of xcorr(rr, reversed source)
 *        (= the causal convolution of rr with the source), low-passed by
 *        fftfilt(fir1(fir_order, fcut / (sr / 2)), .), divided by its
 *        largest magnitude (normalizeIR.m);
 *   t60 = Schroeder integration and the line fit of t60.m on rir.
 * sample_rate <= 0 takes 1 / dt.  rir_out (nt doubles, may be NULL);
 * t60_out (4 doubles, may be NULL): T60 in ms rounded as t60.m returns it,
 * the fitted slope (dB/ms), the fit length `stop`, and 1 when t60.m's
 * window would have been overrun (stop clamped to the window; 0 otherwise).
 * Synchronous. */
int ard_impulse_response(ard_ctx* ctx, int32_t scene, int32_t recorder, int32_t source, int64_t nt,
                         int64_t truncate, double sample_rate, double fcut, int32_t fir_order,
                         double* rir_out, double* t60_out);

/* No counterpart in the reference.  The field readout of ard_read_field for
 * an air partition of an FP32 context, for callers that cannot allocate
 * device memory: it allocates nothing.  The caller passes a device buffer of
 * width*height*depth floats ([z][y][x]), which receives only the finished
 * field; the modes, the transform tables and both intermediates of the
 * transform live in a fixed device array inside the library (44 MiB, on
 * every GPU that loads the library, until exit), so partitions are limited
 * to 4,194,304 cells with every extent at most 1024 (ARD_ERR_RANGE beyond,
 * nothing queued or written).  Asynchronous on `stream` (NULL: the
 * context's stream), ordered after work already queued on the context.  The
 * first call on a device looks up the array's device address and should
 * come before any stream capture.  Calls share the array and it keeps the
 * last call's contents: calls whose work overlaps on the GPU race with each
 * other. */
int ard_read_field_noalloc(ard_ctx* ctx, int32_t scene, int32_t partition, float* out_device, void* stream);

/* ---- adjoint (gradients of a recorder misfit) ---- */

/* Gradients of the recorder misfit
 *   J = 0.5 * sum_{t<T} sum_r (rec[t][r] - target[t][r])^2      (per scene)
 * computed by the hand-written adjoint step run backwards in time.  The
 * call runs the forward itself from the current state, which must be step
 * 0 (ard_reset, then ard_set_initial_pressure as wanted); on return the
 * forward state and the recorder samples are those after step T, as if
 * ard_step(T) had been called.  The context needs options.adjoint.
 * target: T * n_recorders floats per scene ([t][recorder]), concatenated
 * over scenes.  Outputs (any may be NULL), concatenated over scenes:
 *   grad_source  n_sources * T floats per scene ([source][t], the layout of
 *                ard_set_source_series)          dJ/d(source series)
 *   grad_scale   6 floats per scene, ARD_PML_*   dJ/d(PML face scale)
 *   loss         1 float per scene
 * grad_scale needs forward PML values in reverse order.  With
 * checkpoint_every <= 0 the whole PML history is kept when it fits in half
 * the free device memory.  Otherwise (or with checkpoint_every > 0) the run
 * is cut into segments of K steps (K = checkpoint_every, or chosen to
 * balance the memories) swept backwards from the last; for the trailing
 * segments the forward run keeps the interfaces' forcing of the PML strips
 * and the PML state at each segment's start, and the segment's PML runs
 * again on its own before its backward sweep; for the leading segments,
 * where the forcing record does not fit in the free memory, it keeps the
 * whole state at each segment's start and the whole segment runs again.
 * Without grad_scale nothing is stored.  ard_describe names the path taken.
 * dJ/d(initial pressure) of an air partition is read afterwards with
 * ard_read_initial_pressure_grad (width*height*depth floats, [z][y][x]). */
int ard_adjoint(ard_ctx* ctx, int64_t T, const float* target,
                int32_t checkpoint_every,
                float* grad_source, float* grad_scale, float* loss);
int ard_read_initial_pressure_grad(ard_ctx* ctx, int32_t scene, int32_t partition,
                                   float* out);

/* Per-stage device time: runs nsteps steps without graph capture on
 * `stream`, with CUDA events around each kernel, and writes the mean
 * milliseconds per step of each stage into stage_ms[0..7] in launch order:
 * PML update, forward face transform (rows, cols), modal update, recorder
 * sampling, inverse face transform (cols, rows), interface forcing.
 * nstages >= 8.  The steps count as ordinary steps.  Synchronous. */
int ard_profile_steps(ard_ctx* ctx, int64_t nsteps, void* stream, float* stage_ms, int32_t nstages);

/* Message of the last error on this context (NULL ctx: last create error). */
int ard_last_error(const ard_ctx* ctx, char* buf, int64_t n);

/* Introspection, no counterpart in the reference: number of kernels one
 * step launches (the step's CUDA graph holds this many kernel nodes per
 * step, plus one counter kernel per 32 steps). */
int ard_kernels_per_step(const ard_ctx* ctx, int32_t* out);

/* Introspection, no counterpart in the reference: the layout the context
 * uses (modal tiling, face-transform path; with options.autotune, every
 * candidate's measured microseconds per step), as text. */
int ard_describe(const ard_ctx* ctx, char* buf, int64_t n);

/* Library version / ABI check. */
int ard_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ARD_GB300_H */
