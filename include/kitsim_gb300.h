/*
 * kitsim_gb300.h - C ABI of the GB300 (sm_103a) ray-cast-and-accumulate engine.
 *
 * This is the drop-in boundary for kit-sim_daylight's GPU contract: every function below replaces one `gpu_*`
 * function of the reference's `src/internal.h:125-220` (implemented there by `src/gpu.cu` over OptiX and the
 * programs of `src/trace_dev.cu`). The C++ shim `kit-sim_daylight_gb300/shim/daylight_gpu.cpp` implements the
 * reference's `daylight::gpu_*` signatures over these entry points, so the reference's `run.cpp` / `views.cpp`,
 * its C ABI (`daylight_c.h`: DL_DAYLIGHT / DL_VIEWS) and its bindings run unchanged on top of this library.
 *
 * Conventions (the reference's, restated for C):
 *  - Every `int` returning function returns 1 on success and 0 on failure; the message is in kgb_last_error()
 *    (per thread, until the next failing call on that thread). No C++ exception crosses the ABI.
 *  - Host arrays are plain host pointers; the engine owns every device buffer and grows it on demand.
 *  - Layouts on the device follow the reference: visibility bits word-major bits[w*nc + i], transmittance bytes and
 *    view classes / distances direction-major [d*nc + i], reflected-light rows [b*nc + i].
 *  - One engine is used by one thread at a time (the reference's run() is one-at-a-time per process).
 *  - Chunks and launch boundaries change no bit of any result (seeds come from global sensor indices).
 */
#ifndef KITSIM_GB300_H
#define KITSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define KGB_API __declspec(dllexport)
#else
#define KGB_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define KGB_ABI_VERSION 1

/* Ray flags: the bit values of OptiX's OPTIX_RAY_FLAG_* that the reference passes around (gpu_ray_flags /
 * gpu_bounce_flags, src/gpu.cu:739-746; pinned by tests/check_gpu.cpp:98-101 as 5 / 21 / 4 / 20 and 1 / 17). */
#define KGB_RAY_DISABLE_ANYHIT 1u          /* every triangle opaque: visibility bits, no transmittance */
#define KGB_RAY_TERMINATE_ON_FIRST_HIT 4u  /* any-hit occlusion (the visibility pass) */
#define KGB_RAY_CULL_BACK_FACING 16u       /* one-sided occluders: back-facing hits are ignored */

/* Slot flags (src/params.h:13-19). */
#define KGB_SLOT_GLASS 1u   /* transmittance by angle (Radiance glass); else tau at every angle */
#define KGB_SLOT_THIN 2u    /* closed thin solid: its exit face passes everything */
#define KGB_SLOT_INWARD 4u  /* ... wound inward: entry is the back face */
#define KGB_SLOT_TWIN 8u    /* ... of no volume, faces in coincident pairs */

/* Views: label of a triangle rays pass, most panes passed, class bit of a ray that passed glass (src/params.h:22-24). */
#define KGB_LABEL_PASS 255u
#define KGB_MAX_PANES 16u
#define KGB_VIEW_GLAZED 0x80u
#define KGB_VIEW_CLASSES 19u /* sky, ground, obstruction, 16 target groups (src/gpu.cu:48) */

/* Optics of one global slot: the reference's Slot (src/params.h:7-12), same layout. */
typedef struct kgb_slot {
  float rho;      /* diffuse reflectance (bounce pass) */
  float tau;      /* transmittance at normal incidence; > 0 = translucent */
  float tn;       /* glass transmissivity (tn_from_Tn(tau)), used with KGB_SLOT_GLASS */
  uint32_t flags; /* KGB_SLOT_* */
} kgb_slot;

typedef struct kgb_engine kgb_engine;

/* A built scene (BVH, triangles, per-triangle slots) moved out of an engine: the reference's GasSlot
 * (src/internal.h:141). */
typedef struct kgb_scene {
  void* handle;
  uint64_t bytes;
} kgb_scene;

/* The reference's GpuStats (src/internal.h:211-216). */
typedef struct kgb_stats {
  double buildMs, traceMs, bounceMs;
  uint64_t rays, gasBytes, launches, paths, bounceLaunches;
  uint64_t buildTempBytes, buildOutputBytes;
  double seriesMs;          /* device time of the tensor-core series kernels (CUDA events), summed over calls */
  uint64_t seriesOutputs;   /* outputs those kernels wrote (sensors x steps), summed */
} kgb_stats;

/* Cancel hook: returns non-zero once the run should stop (the reference's const std::atomic<bool>*). */
typedef int (*kgb_cancel_fn)(void* ctx);

/* Inputs of kgb_series: the reference's SeriesIn (src/internal.h:155-168), host arrays. */
typedef struct kgb_series_in {
  uint32_t nSky;          /* sky directions are 0..nSky-1 */
  const int32_t* row;     /* [nSky] patch index per sky direction */
  const float* wsky;      /* [nSky] weight per sky direction */
  const float* S;         /* [P x T] patch radiance per step, row-major */
  int32_t P, T;
  const float* g;         /* [T] ground term per step */
  const float* G;         /* [nc] ground visibility per sensor */
  uint32_t sun0, nSun;    /* sun direction range in the direction table */
  const int32_t* sunStep; /* [nSun] step (column) index per sun direction */
  const float* sunVec;    /* [nSun x 3] */
  const float* sunW;      /* [nSun] DNI (W/m2) or direct illuminance (lux) per sun direction */
  const float* Sdc;       /* [(P+1) x T] radiance per bounce bin and step; NULL = no reflected light */
} kgb_series_in;

/* Inputs of kgb_bounce: the reference's Bounce (src/internal.h:178). */
typedef struct kgb_bounce_in {
  uint32_t N;      /* diffuse reflections per path */
  uint32_t M;      /* paths per sensor */
  int32_t mf;      /* sky density of the bins (1, 2, 4) */
  double north;    /* degrees */
  kgb_cancel_fn cancel;
  void* cancelCtx;
} kgb_bounce_in;

/* Inputs of kgb_view: the reference's ViewLaunch (src/internal.h:186-195). */
typedef struct kgb_view_in {
  uint32_t nAz, nEl;
  float az0, dAz;        /* degrees */
  const float* rowSin;   /* [2 nEl] host: sin of each row's bottom and top elevation */
  int32_t world, cull, jitter, back, vground;
  uint32_t nS;           /* sides per element */
  float groundZ;         /* the virtual ground plane (recentred) */
  double north;          /* degrees */
  kgb_cancel_fn cancel;
  void* cancelCtx;
} kgb_view_in;

/* --- lifetime -------------------------------------------------------------------------------------------------- */
KGB_API int32_t kgb_version(void);
KGB_API const char* kgb_last_error(void);
/* replaces gpu_init (src/internal.h:127): the engine on the current CUDA device; NULL + kgb_last_error on failure */
KGB_API kgb_engine* kgb_init(void);
/* replaces gpu_destroy (src/internal.h:128) */
KGB_API void kgb_destroy(kgb_engine* e);

/* --- scene --------------------------------------------------------------------------------------------------------- */
/* replaces gpu_build (src/internal.h:133): v [nv x 3] floats, tri [nt x 3] vertex indices, slot [nt] global slot per
 * triangle (NULL when not needed), the slot table. Builds the 8-wide BVH; every slot index must be < nSlots when the
 * build is slotted (a slot transmits or perSlot). nt == 0: an empty scene, every ray misses. */
KGB_API int kgb_build(kgb_engine* e, const float* v, size_t nv, const uint32_t* tri, size_t nt, const uint32_t* slot,
                      const kgb_slot* slots, size_t nSlots, int perSlot);
/* replaces gpu_build_bytes (src/internal.h:136): device bytes a build peaks at; UINT64_MAX on error */
KGB_API uint64_t kgb_build_bytes(kgb_engine* e, size_t nv, size_t nt, int slotted);
/* replaces gpu_trim (src/internal.h:138) */
KGB_API void kgb_trim(kgb_engine* e, int sensors);
/* replaces gpu_set_slots (src/internal.h:139): the slot records read at hits (tau, tn, rho, flags) */
KGB_API int kgb_set_slots(kgb_engine* e, const kgb_slot* slots, size_t n);
/* replace gpu_detach / gpu_attach / gpu_free / gpu_free_bytes (src/internal.h:142-145) */
KGB_API kgb_scene kgb_detach(kgb_engine* e);
KGB_API void kgb_attach(kgb_engine* e, kgb_scene s);
KGB_API void kgb_free_scene(kgb_scene* s);
KGB_API uint64_t kgb_free_bytes(void);
/* replaces gpu_set_scene (src/internal.h:146): resident sensors (recentred, offset applied) and directions. The
 * visibility traces take a call's sensors grouped by the orientation of their normals (each sensor's result, and where
 * it is written, do not change); that order is rebuilt here when the sensors' orientation classes differ from those it
 * was built from (checked on the device), so resending the same sensors costs one small kernel. */
KGB_API int kgb_set_scene(kgb_engine* e, const float* P, const float* N, size_t nSensors, const float* D, size_t nDir);
/* replaces gpu_set_labels (src/internal.h:197): class per triangle in build order; n == 0: none */
KGB_API int kgb_set_labels(kgb_engine* e, const uint8_t* label, size_t n);

/* --- daylight -------------------------------------------------------------------------------------------------------- */
/* replaces gpu_trace (src/internal.h:151): sensors [i0, i0+nc) against every direction. Without
 * KGB_RAY_DISABLE_ANYHIT: transmittance bytes instead of bits. */
KGB_API int kgb_trace(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags);
/* replaces gpu_reduce (src/internal.h:154): out[i] = sum_d T(i,d) * (useCos ? max(0, N_i.D_d) : 1) * W[d] (double) */
KGB_API int kgb_reduce(kgb_engine* e, size_t nc, const float* W, int useCos, double* out);
/* No counterpart in the reference. kgb_reduce for a caller that must not allocate device memory at the time of the
 * call: a host that reserved the GPU's memory for its own pool up front, or a plugin host that forbids device
 * allocation once its processing loop runs (a failed or extra cudaMalloc there breaks the host). Same arguments,
 * kernels and results as kgb_reduce, bit for bit; the weights and the sums are staged in one fixed 1 MiB array of
 * device memory that belongs to the library (every GPU that loads the library holds it until the process exits)
 * instead of in engine buffers that kgb_reduce may have to grow. Limit: nDir weights (4 bytes each, rounded up to
 * 256 bytes) plus nc sums (8 bytes each) must fit in 1 MiB, e.g. at most 128,256 sensors per call with 5610
 * directions; a larger call fails with a message giving the limit. The first call on a device looks the array's
 * address up (cudaGetSymbolAddress): make that first call before any stream capture. Every call uses the same
 * array, so calls whose work overlaps on the GPU (other threads, other engines on the device) race; each call waits
 * for its own work before it returns. Nothing in the array needs clearing between calls: the weights are copied in
 * and every sum is written before it is read. */
KGB_API int kgb_reduce_noalloc(kgb_engine* e, size_t nc, const float* W, int useCos, double* out);
/* replaces gpu_series (src/internal.h:171): E[i*T + t] (host, nc x T floats) */
KGB_API int kgb_series(kgb_engine* e, size_t nc, const kgb_series_in* in, float* E);
/* gpu_series followed by the reference's fwrite of E into the --timeseries .npy (src/run.cpp:683-686), in one call:
 * the same rows written to the open file fd at byte offset (its header's length + i0 x T x 4 for the chunk that starts
 * at sensor i0), straight from the engine's pinned staging, while the next rows come down */
KGB_API int kgb_series_file(kgb_engine* e, size_t nc, const kgb_series_in* in, int fd, uint64_t offset);
/* replaces gpu_bounce (src/internal.h:179) */
KGB_API int kgb_bounce(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_bounce_in* b);
/* replaces gpu_reduce_dc (src/internal.h:180): out[i] = sum_b dc(b, i) * W[b] (double) */
KGB_API int kgb_reduce_dc(kgb_engine* e, size_t nc, const float* W, double* out);
/* replace gpu_download_dc / bits / bytes (src/internal.h:181-183): count must be the buffer's element count */
KGB_API int kgb_download_dc(kgb_engine* e, size_t nc, float* out, size_t count);
KGB_API int kgb_download_bits(kgb_engine* e, size_t nc, uint32_t* out, size_t count);
KGB_API int kgb_download_bytes(kgb_engine* e, size_t nc, uint8_t* out, size_t count);

/* --- views ----------------------------------------------------------------------------------------------------------- */
/* replaces gpu_view (src/internal.h:201): launch carries the sub-launch size from chunk to chunk (0 = start over) */
KGB_API int kgb_view(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, const kgb_view_in* v, size_t* launch);
/* replaces gpu_reduce_view (src/internal.h:208): out [nc x NA] doubles,
 * NA = 3 nClass + 1 + nReach + (glazing ? 1 : 0) + (isoDim ? 1 : 0) */
KGB_API int kgb_reduce_view(kgb_engine* e, size_t nc, const double* wRow, size_t nRow, uint32_t nClass, double farDist,
                            const float* reach, size_t nReach, int glazing, uint32_t isoDim, double* out);
/* replaces gpu_download_view (src/internal.h:210): [nc x K] each (transposed from the device's [K x nc] on the device) */
KGB_API int kgb_download_view(kgb_engine* e, size_t nc, uint8_t* cls, float* dist, size_t count);
/* the last trace's visibility as one row per sensor, transposed on the device: [nc x nWords] words (bits) or
 * [nc x nDir] bytes; they replace gpu_download_bits / gpu_download_bytes plus the host transposes of the reference's
 * --dump-bits (src/run.cpp:659-671) */
KGB_API int kgb_download_bits_rows(kgb_engine* e, size_t nc, uint32_t* out, size_t count);
KGB_API int kgb_download_bytes_rows(kgb_engine* e, size_t nc, uint8_t* out, size_t count);

/* --- misc ------------------------------------------------------------------------------------------------------------ */
/* replaces gpu_stats (src/internal.h:216) */
KGB_API kgb_stats kgb_get_stats(const kgb_engine* e);
/* replace gpu_ray_flags / gpu_bounce_flags (src/internal.h:218-220) */
KGB_API uint32_t kgb_ray_flags(int cullBackfaces, int translucent);
KGB_API uint32_t kgb_bounce_flags(int cullBackfaces);
/* Sizes of the engine's current buffers (no reference counterpart; what a C caller needs to size downloads):
 * out[0] = nSensors, out[1] = nDir, out[2] = nWords, out[3] = nBins (last bounce), out[4] = K (last view),
 * out[5] = 1 when the last trace wrote bytes. */
KGB_API void kgb_dims(const kgb_engine* e, uint64_t out[6]);

/* --- scene preparation (the reference's host code beside its GPU contract, here on the GPU) ------------------------ */
/* replaces triangulate_into (src/mesh.cpp:137-168; scene_acquire calls it per mesh): one mesh's faces as triangles.
 * points [nPoints x 3] doubles, counts [nFaces] corners per face, indices [sum of counts], faceSlot [nFaces] the face's
 * optics slot (NULL: 0), c [3] the centre the scene is recentred on. Writes v [nPoints x 3] floats (each point minus c),
 * tri [capacity x 3] (vertex indices + base) and slot [capacity] (slotBase + the face's slot; NULL: none), capacity =
 * sum over faces of max(0, corners - 2); triangles in face order: a triangle as given, a quad as 0-1-2 and 0-2-3, five or
 * more corners by ear clipping on the face's Newell plane (include/kgb_earcut.h, mapbox earcut's algorithm, at most
 * corners - 2 of them). *made: the triangles written; *skipped: the faces that gave none (fewer than 3 corners, no
 * area, or no ear). */
KGB_API int kgb_triangulate(kgb_engine* e, const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices,
                            const uint32_t* faceSlot, const double* c, uint32_t base, uint32_t slotBase, float* v, uint32_t* tri, uint32_t* slot,
                            size_t* made, int32_t* skipped);
/* replaces thin_solid (src/mesh.cpp:275-304) for every slot of a mesh at once: flags[s] (s < nSlots) = KGB_SLOT_THIN,
 * with KGB_SLOT_TWIN (no volume: twice the volume over the area under 1e-5 m) or KGB_SLOT_INWARD (negative volume), when
 * slot s's faces weld (0.01 mm grid, recentred on c) into a closed surface (every directed edge matched by its reverse)
 * with twice the volume over the area under 0.1 m; else 0. */
KGB_API int kgb_thin_solids(kgb_engine* e, const double* points, size_t nPoints, const int32_t* counts, size_t nFaces, const int32_t* indices,
                            const uint32_t* faceSlot, uint32_t nSlots, const double* c, uint32_t* flags);

/* --- meshes read straight to the device (the reference reads them into host vectors) ------------------------------- */
/* A .dmesh image (the reference's format, src/daylight.h:129-136: "DLM1", u32 flags (bit 0: a slot block), u64 nPoints,
 * nFaces, nIndices; then float64 xyz points, int32 counts, int32 0-based indices, and with bit 0 one uint16 slot per
 * face; little-endian, no padding) held by the engine on the device after the reference's checks. */
typedef struct kgb_mesh_info {
  uint32_t id;          /* the mesh's handle in this engine; KGB_NO_MESH when the image holds no faces (nothing is kept:
                           the reference drops an empty mesh, src/mesh.cpp:472) */
  uint32_t slots;       /* slot_count (src/mesh.cpp:170): 1 + the largest face slot, 1 without a slot block */
  uint64_t nPoints, nFaces, nIndices;
  uint32_t hasSlots;    /* the image had the slot block */
  uint32_t maxCorners;  /* the largest face's corner count */
  uint64_t triCap;      /* tri_cap (src/mesh.cpp:120-124): the sum over faces of corners - 2 */
  double lo[3], hi[3];  /* the points' bounds, fmin / fmax per axis as bbox_centre takes them (src/mesh.cpp:107-118);
                           +inf / -inf without points */
} kgb_mesh_info;
#define KGB_NO_MESH 0xffffffffu
/* replaces read_dmesh(data, size, name, ...) (src/mesh.cpp:476-478 over parse_dmesh, 450-474): one image in host
 * memory. The 32-byte header is checked on the host; the arrays are copied to the device (straight from page-locked
 * memory, else through pinned slices) and checked there by the reference's rules (mesh_ok, src/mesh.cpp:436-445: faces
 * of 3 or more corners, the counts summing to nIndices, every index within the points). A failure gives the reference's
 * message, `name` first ("NAME: truncated", "NAME: vertex index out of range", ...). The engine keeps the arrays, with
 * each face's first index, until kgb_mesh_free or kgb_destroy. Points, faces and indices beyond 2^32 - 1 are refused. */
KGB_API int kgb_mesh_read(kgb_engine* e, const void* data, size_t size, const char* name, kgb_mesh_info* info);
/* replaces read_dmesh(path, ...) (src/mesh.cpp:480-489): the file read in 32 MiB slices into two pinned buffers, each
 * slice copied to the device while the next one is read; the checks and messages as kgb_mesh_read's, with the path as
 * the name ("cannot open PATH", "PATH: truncated", ...). */
KGB_API int kgb_mesh_file(kgb_engine* e, const char* path, kgb_mesh_info* info);
/* A kept mesh's arrays back to the host (each pointer may be NULL; slot only when the image had the slot block). */
KGB_API int kgb_mesh_download(kgb_engine* e, uint32_t id, double* points, int32_t* counts, int32_t* indices, uint16_t* slot);
KGB_API int kgb_mesh_free(kgb_engine* e, uint32_t id);
/* kgb_thin_solids on a kept mesh: flags [info.slots], its faces' slots as the image gives them. */
KGB_API int kgb_mesh_thin_solids(kgb_engine* e, uint32_t id, const double* c, uint32_t* flags);
/* replaces the scene assembly of scene_acquire (src/run.cpp:98-150) and its gpu_build, for kept meshes: no array of the
 * scene passes through the host. Meshes ids[0 .. nMeshes) in the run's order; blocks[k] (NULL: all) whether mesh k
 * blocks rays. As run.cpp lays it out: the points of the blocking meshes one after the other, recentred on c (the
 * caller's bbox_centre over the infos' lo / hi); slot bases over every mesh, each mesh taking its info.slots; the
 * triangles of the blocking meshes in mesh order, each mesh's faces triangulated as kgb_triangulate does, with its
 * vertex base and slot base. The scene is then built as kgb_build builds it from those arrays (slots / nSlots /
 * perSlot as there). made [nMeshes] (may be NULL): each mesh's triangles (0 for one that does not block); *skipped
 * (may be NULL): the faces that gave none. */
KGB_API int kgb_build_meshes(kgb_engine* e, const uint32_t* ids, size_t nMeshes, const uint8_t* blocks, const double* c, const kgb_slot* slots,
                             size_t nSlots, int perSlot, uint64_t* made, int32_t* skipped);

/* --- sky (no C ABI counterpart in the reference: it builds its sky on the host) ---------------------------------- */
/* One time step of the sky model, the inputs of the reference's gendaymtx_step (src/sky.cpp:297): day of year (as
 * gendaymtx computes it), sun altitude and azimuth (radians, azimuth clockwise from north), DNI and DHI (W/m2). */
typedef struct kgb_sky_step {
  int32_t jd, pad;
  double alt, azi, dni, dhi;
} kgb_sky_step;
/* The Perez all-weather sky + AddDirect of T steps at sky density mf (1, 2, 4) on the GPU in FP64, restating
 * gendaymtx_step (src/sky.cpp:297-474, called per step by src/run.cpp:372-446): out [T x 3 (P + 1)] floats, each step's
 * row as gendaymtx_step writes it (ground first, then the patches; RGB). sun / sky / visible as its flags. */
KGB_API int kgb_sky(kgb_engine* e, int32_t mf, const kgb_sky_step* steps, size_t T, double grefl, int32_t sun, int32_t sky,
                    int32_t visible, float* out);
/* Ladybug mode's sky on the GPU (the reference's --mode ladybug, src/run.cpp:362-398 and 447-470: gendaymtx -A as
 * ladybug runs it). steps [T x 4]: day of year (gendaymtx's jd), hour (decimal, the weather's clock), DNI, DHI (W/m2, as
 * the steps hold them: truncated to integers here as ladybug's .wea prints them); lat, lon (degrees, east positive) and
 * tz (hours east of UTC) of the weather, printed into the .wea as ladybug does (0.01 degree, the zone's integer
 * meridian); grefl; durationHours (the steps' total hours). Per step the sun by Radiance's sun.c and the Perez sky twice
 * (sun alone, sky alone), FP64 on the GPU; per patch the float sums over all steps in step order; their averages printed
 * to three significant digits (%.3g) on the host. Writes lb [3 P + 1] doubles: per patch skyDirLB, then skyDifLB, then
 * skyRad (their sum), then gndLB: the values run.cpp puts into its weight vectors (direct, diffuse, radiation; ground).
 * acc [4 P + 6] floats, when non-null: the sums (red of the sun rows [P], the sky rows [3 P], the ground row of the sun
 * rows [3] and of the sky rows [3]). S [P x Tup], g [Tup], when non-null: the series columns of the steps with
 * DNI + DHI > 1e-4 (run.cpp:385-397). mf 1 or 2 (the reference's rule for ladybug mode). */
KGB_API int kgb_sky_ladybug(kgb_engine* e, int32_t mf, const double* steps, size_t T, double lat, double lon, double tz, double grefl,
                            double durationHours, double* lb, float* acc, float* S, float* g);
/* NOAA solar positions of T steps on the GPU in FP64, restating sun_noaa (src/solar.cpp:66-105): in [T x 7] = lat, lon,
 * tz, month, day, hour (decimal), leap; out [T x 6] = altitude (deg, refracted), azimuth (deg), up, direction x y z. */
KGB_API int kgb_sun_noaa(kgb_engine* e, const double* in, size_t T, double* out);

/* --- serving (no reference counterpart: the reference runs one request at a time, src/run.cpp:35) ---------------- */
/* A server keeps scenes resident and runs daylight and views requests of any size with continuous batching: requests
 * are admitted as the HBM budget allows and cut into work items that run back to back on one stream, two queued at a
 * time, picked by a priority (requests waiting over 1.2 s first, in arrival order; the others by remaining work over
 * age plus 0.3 s): daylight batches packing chunks of any number of
 * requests (one persistent any-hit launch + one multi-quantity reduce, a CUDA graph) and views chunks (the view
 * kernels on a range of one request's sensors). Results equal the single-request entry points' bit for bit. A
 * request's host arrays must stay valid until kgb_server_wait returns for it. */
typedef struct kgb_server kgb_server;
typedef struct kgb_daylight_request {
  int32_t scene;
  uint32_t nSensors, nDir, nQ; /* nQ quantities, 1..8 */
  const float* P;              /* [nSensors x 3] recentred sensor points (offset applied) */
  const float* N;              /* [nSensors x 3] unit normals */
  const float* D;              /* [nDir x 3] directions */
  const float* W;              /* [nQ x nDir] weights per quantity (gpu_reduce's W) */
  uint32_t useCosMask;         /* bit q: quantity q weighted by max(0, N.D) */
  uint32_t rayFlags;           /* visibility bits: KGB_RAY_DISABLE_ANYHIT set */
  double* out;                 /* [nQ x nSensors] sums, as gpu_reduce gives them */
} kgb_daylight_request;
typedef struct kgb_views_request {
  int32_t scene;
  uint32_t nSensors;
  const float* P;
  const float* N;
  const uint8_t* label;        /* [scene triangles] classes, or NULL (every hit an obstruction) */
  kgb_view_in view;            /* the grid; its cancel hook is not used */
  uint32_t rayFlags;
  const double* wRow;          /* [nEl] */
  uint32_t nClass;
  double farDist;
  const float* reach;
  uint32_t nReach;
  int32_t glazing;
  uint32_t isoDim;
  double* out;                 /* [nSensors x NA], gpu_reduce_view's columns */
} kgb_views_request;
/* A daylight request's hourly time series (the reference's --timeseries: gpu_series per chunk, src/run.cpp:672-687,
 * src/gpu.cu:639-669), computed inside the server's daylight batches: in.* as for kgb_series (nSky, row, wsky, S, P, T,
 * g, sun0, nSun, sunStep, sunVec, sunW; G and Sdc must be NULL: G is the request's quantity gQ, its sums as float, as
 * run.cpp passes its ground reduce; the server has no reflected light). Every batch's series chunks, of any number of
 * requests, run as ONE grouped split-BF16 tensor-core launch (at most 48 chunks), the rows of E bit-identical to
 * kgb_series' tensor-core form on the same inputs. One sun direction per step (the tensor-core form's sun term). */
typedef struct kgb_series_request {
  kgb_series_in in;
  uint32_t gQ;   /* the quantity of the request whose sums give G */
  float* E;      /* [nSensors x T] out */
} kgb_series_request;
KGB_API kgb_server* kgb_server_create(uint64_t hbmBudgetBytes);
KGB_API void kgb_server_destroy(kgb_server* s);
/* a resident scene (8-wide BVH) for requests; *sceneId its index */
KGB_API int kgb_server_add_scene(kgb_server* s, const float* v, size_t nv, const uint32_t* tri, size_t nt, int32_t* sceneId);
/* times calibration batches on scene 0 and keeps the fastest chunk and batch sizes (call while idle) */
KGB_API int kgb_server_autotune(kgb_server* s);
/* sets by hand what the autotuner picks (call while idle; 0 keeps a value): sensors per daylight chunk (32..2^20), rays
 * per daylight batch (2^16..2^32) and rays per views chunk (2^16..2^31, default 2^27) */
KGB_API int kgb_server_set_tuning(kgb_server* s, uint32_t chunkSensors, uint64_t batchRays, uint64_t viewRays);
/* the scheduler's priority: a request that has waited more than oldSeconds goes first, in arrival order; the others by
 * their remaining work divided by (their age + ageSeconds). Defaults 1.0 s and 0.3 s; takes effect at the next pick. */
KGB_API int kgb_server_set_priority(kgb_server* s, double oldSeconds, double ageSeconds);
/* out[3]: the tuning in use (autotuned or set by hand): sensors per daylight chunk, rays per daylight batch, rays per
 * views chunk */
KGB_API void kgb_server_tuning(kgb_server* s, uint64_t* out);
KGB_API int kgb_server_submit(kgb_server* s, const kgb_daylight_request* r, uint64_t* ticket);
KGB_API int kgb_server_submit_views(kgb_server* s, const kgb_views_request* r, uint64_t* ticket);
/* a daylight request that also gives its time series (its host arrays, the series' included, valid until it is waited
 * for) */
KGB_API int kgb_server_submit_series(kgb_server* s, const kgb_daylight_request* r, const kgb_series_request* q, uint64_t* ticket);
/* 1 once the request completed (its out written), 0 on failure or timeout (kgb_last_error) */
KGB_API int kgb_server_wait(kgb_server* s, uint64_t ticket, double timeoutSec);
/* out[10]: completed requests, latency p50, p90, p99, max (s), rays, work items (daylight batches and views chunks), HBM
 * bytes in use, chunk sensors, batch rays */
KGB_API void kgb_server_stats(kgb_server* s, double* out);
/* out[5]: GPU seconds and rays of daylight batches, the same of views chunks (events around each item on the work
 * stream), and wall seconds with work queued on it */
KGB_API void kgb_server_timing(kgb_server* s, double* out);

/* --- no reference counterpart ---------------------------------------------------------------------------------- */
/* The CUDA stream (a cudaStream_t) the engine's work runs on from now on; NULL: the engine's own stream. Calls still
 * return after their work is done; a caller times them with events on this stream. */
KGB_API int kgb_set_stream(kgb_engine* e, void* stream);
/* The form kgb_series computes in: 0 (default) the split-BF16 contraction on the tensor cores (tcgen05, FP32
 * accumulation, the sun term in FP32), 1 the plain FP32 form (one thread per sensor, the reference's k_series
 * restated), kept as the measured baseline. */
KGB_API int kgb_set_series_form(kgb_engine* e, int form);
/* No counterpart in the reference (its gpu_build builds an OptiX GAS on the device): which builder the following
 * kgb_build calls use. 1 (the default): on the device, a Morton-ordered radix tree (LBVH) refined by treelet
 * restructuring, collapsed to 8-wide nodes; 0: a binned-SAH binary tree built on the host, collapsed the same way.
 * Every result is the same either way (both trees are conservative); the device builder is 15x faster on 2 M
 * triangles and its tree traces about as fast. */
KGB_API int kgb_set_builder(kgb_engine* e, int which);
/* No counterpart in the reference: lowers the bounded-execution limits of the following calls, so that tests can drive
 * them to their error returns. nodeLimit: the traversals of kgb_trace, kgb_view and kgb_bounce see only the BVH's first
 * nodeLimit nodes, and so at most nodeLimit + 8 node visits per query; a query that needs more gives up and the call
 * fails ("traversal gave up ...", the message of a walk past its visit cap; 0: every node, the cap then the node count
 * + 8, at most 2^20). bounceLimitNs: how long one bounce step kernel may run before it ends its remaining paths and
 * kgb_bounce fails ("... passed its ... limit ..."; 0: the default, 10 s; larger values are clamped to it).
 * seriesWaitNs: how long a wait of the tensor-core series pipeline (its producer, MMA issuer and epilogue on their
 * mbarriers) may last before the kernel records a timeout, finishes the copies and MMAs it issued, frees its TMEM and
 * ends, and kgb_series fails ("... timed out waiting ..."; 0: the default, 4 s; larger values are clamped to it).
 * flags: KGB_LIMIT_WITHHOLD_FILLS makes the series pipeline's producer issue no shared-memory fills, so that its waits
 * run out for certain (a barrier nothing completes): the test of that path. The engine stays usable after any of
 * these failures. */
#define KGB_LIMIT_WITHHOLD_FILLS 1u
KGB_API int kgb_set_limits(kgb_engine* e, uint32_t nodeLimit, uint64_t bounceLimitNs, uint64_t seriesWaitNs, uint32_t flags);
/* Instrumentation for the traversal roofline: traces sensors [i0, i0+nc) exactly as kgb_trace does (same bits / bytes
 * left on the device) with counting kernels, out[0] = BVH nodes visited, out[1] = triangles tested, out[2] = rays
 * traced past the hemisphere cull, out[3] = BVH bytes (nodes + triangle records). */
KGB_API int kgb_trace_counters(kgb_engine* e, size_t i0, size_t nc, uint32_t rayFlags, uint64_t out[4]);

#ifdef __cplusplus
}
#endif
#endif /* KITSIM_GB300_H */
