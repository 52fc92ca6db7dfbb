/*
 * drr_gb300.h -- C ABI of the GB300-native DeepDRR volume projector (libdrr_gb300.so).
 *
 * The library renders digitally reconstructed radiographs of one or more CT volumes: a fixed-step
 * ray march with trilinear density sampling and per-material label fractions, followed by
 * polychromatic Beer-Lambert attenuation over an X-ray spectrum. All entry points are plain C:
 * handles, host pointers for small per-view geometry, device pointers for volumes and images, and
 * a CUDA stream. No torch types cross this boundary.
 *
 * Each entry point replaces a piece of the reference projector (deepdrr v1.2.2):
 *   drr_volset_create   Projector.initialize texture setup, deepdrr/projector/projector.py:1464-1546
 *                       and create_cuda_texture, projector.py:116-257
 *   drr_tables_create   the spectrum / mass-attenuation upload of Projector.initialize,
 *                       projector.py:1659-1686
 *   drr_project         Projector._render_single + _update_object_locations + the projectKernel
 *                       launch, projector.py:709-800, 802-831; kernel deepdrr/projector/project_kernel.cu:135-650
 *   drr_*_destroy       Projector.free, projector.py:1719-1764
 *   drr_ingest_hu       Volume.from_hu's HU conversion and thresholding, deepdrr/vol/volume.py:281-351
 *   drr_mesh_*          the reference's OpenGL mesh passes (pyrenderdrr) read by project_kernel.cu
 *   drr_add_noise       analytic_generators.add_noise, deepdrr/projector/analytic_generators.py:10-18
 *   drr_clip_upper,     the post-processing of Projector.project, projector.py:697-702, and
 *   drr_neglog          deepdrr/utils/image_utils.py:18-58
 * and adds what the reference does not have: persistent multi-view launches, their CUDA-graph
 * capture and launch-shape autotuner (drr_graph_*, drr_autotune), and the adjoint
 * (drr_project_adjoint, drr_volset_set_density) for density and pose gradients.
 *
 * Conventions. Volumes are stored i-fastest ([nk][nj][ni]), i.e. the reference's
 * np.moveaxis(data, [0,1,2], [2,1,0]) layout (projector.py:1469). Images are row-major [H][W]
 * (the reference kernel writes column-major and the host transposes, projector.py:786-792).
 * Every call is stream-ordered on the stream it is given; a handle must not be used from two
 * host threads at once without external synchronisation. Errors are returned as status codes and
 * described by drr_last_error() (thread-local); no kernel traps.
 */
#ifndef DRR_GB300_H
#define DRR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DRR_OK = 0,
    DRR_ERR_INVALID_ARGUMENT = 1, /* the reference raises ValueError / AssertionError here */
    DRR_ERR_UNSUPPORTED = 2,      /* a size or mode the library does not implement */
    DRR_ERR_CUDA = 3,             /* a CUDA runtime call failed; see drr_last_error() */
    DRR_ERR_OUT_OF_MEMORY = 4
} drr_status;

typedef enum {
    DRR_DENSITY_F32 = 0, /* float32 densities, hardware-filtered like the reference */
    DRR_DENSITY_F16 = 1, /* IEEE half densities, hardware-filtered, float32 accumulation */
    DRR_DENSITY_BF16 = 2 /* bfloat16 densities, held exactly in a float16 texture (values 0 or with |x| in
                            [2^-14, 65504]; others are rejected), float32 accumulation */
} drr_density_type;

#define DRR_MAX_VOLUMES 4
#define DRR_MAX_MATERIALS 16

/* One CT volume. `density` and `labels` are DEVICE pointers owned by the caller; the library
 * copies them into its own texture storage during drr_volset_create and does not keep them. */
typedef struct {
    const void *density;    /* [nk][nj][ni] of drr_density_type */
    const uint8_t *labels;  /* [nk][nj][ni], material index into the projector's sorted material list */
    int32_t ni, nj, nk;
    int32_t density_type;   /* drr_density_type */
} drr_volume_desc;

typedef struct drr_volset drr_volset;
typedef struct drr_tables drr_tables;

/* Create the device-side copy of `n_volumes` volumes (textures) for an `n_materials` projector.
 * Labels are checked on the device to be < n_materials. Synchronous with respect to `stream`.
 * Replaces projector.py:1464-1546 (texture creation) and create_cuda_texture, projector.py:116-257. */
drr_status drr_volset_create(const drr_volume_desc *volumes, int32_t n_volumes, int32_t n_materials,
                             void *stream, drr_volset **out);
drr_status drr_volset_destroy(drr_volset *set);

/* Replace the densities of volume `volume` from a device array of the type and size it was created
 * with ([nk][nj][ni], i fastest), asynchronously on `stream` (float32 and float16 volumes; a
 * bfloat16 volume returns DRR_ERR_UNSUPPORTED). Labels are kept. No counterpart in the reference:
 * it lets a differentiable caller project the current iterate without rebuilding the set. */
drr_status drr_volset_set_density(drr_volset *set, int32_t volume, const void *density, void *stream);

typedef enum {
    DRR_HU_F32 = 0, /* float32 Hounsfield units (converted in float32, as numpy does) */
    DRR_HU_I16 = 1, /* int16 Hounsfield units (converted in float64, then rounded to float32) */
    DRR_HU_F64 = 2  /* float64 Hounsfield units (likewise) */
} drr_hu_type;

/* Volume ingest on the GPU: replaces the numpy work of Volume.from_hu (deepdrr/vol/volume.py:281-302:
 * _convert_hounsfield_to_density, volume.py:339-351, and the thresholding of load_dicom.py:132-143)
 * and the i-fastest layout change of projector.py:1469. `hu` is a DEVICE array [ni][nj][nk] (k
 * fastest, the reference's layout); `density` (drr_density_type, float32 / float16 / bfloat16 rounded
 * to nearest) and `labels` are DEVICE arrays [nk][nj][ni] ready for drr_volume_desc. class_labels
 * (host) are the labels written for air (HU <= -800), soft tissue (-800 < HU <= 350) and bone
 * (HU > 350); NaN HU are air. Asynchronous on `stream`. */
drr_status drr_ingest_hu(const void *hu, int32_t hu_type, int32_t ni, int32_t nj, int32_t nk,
                         const uint8_t class_labels[3], void *density, int32_t density_type, uint8_t *labels,
                         void *stream);

/* Upload a spectrum and its mass-attenuation table. Host pointers:
 *   energies_kev [n_bins], pdf [n_bins], mu_over_rho [n_bins][n_materials] (cm^2/g).
 * Replaces projector.py:1659-1686. */
drr_status drr_tables_create(const float *energies_kev, const float *pdf, const float *mu_over_rho,
                             int32_t n_bins, int32_t n_materials, void *stream, drr_tables **out);
drr_status drr_tables_destroy(drr_tables *tables);

enum {
    DRR_FLAG_ATTENUATE_OUTSIDE = 1 << 0, /* Projector(attenuate_outside_volume=True), project_kernel.cu:358-361,522-527,557-560 */
    DRR_FLAG_FULL_MARCH = 1 << 1,        /* march every step from minAlpha like the reference (no prefix skip); for testing */
    DRR_FLAG_PERSISTENT = 1 << 2         /* one persistent launch for all views (dynamic (view, tile) scheduling) */
};

/* Arguments of one drr_project call: `n_views` views of the same volume set. `struct_size` must be
 * sizeof(drr_project_args) as the caller's binding lays the struct out (e.g.
 * `drr_project_args a = {sizeof(drr_project_args)};`); any other value is rejected with
 * DRR_ERR_INVALID_ARGUMENT before any other field is read, so a binding whose copy of this struct
 * has drifted from the library's fails loudly instead of having fields read past its end. */
typedef struct {
    uint32_t struct_size;           /* sizeof(drr_project_args) */
    int32_t width, height;          /* detector size in pixels */
    float step;                     /* ray step in world units (mm), Projector(step=...) */
    float max_ray_length;           /* <= 0: unlimited; projector.py:641-650 */
    int32_t air_index;              /* index of "air" in the sorted material list (attenuate flag) */
    uint32_t flags;                 /* DRR_FLAG_* */
    int32_t n_views;
    const int32_t *priority;        /* host [n_volumes]; smaller number wins (projector.py:489-500) */
    const int32_t *enabled;         /* host [n_volumes]; 0 = volume ignored */
    const double *world_from_index; /* host [n_views][3][3]: ray(u,v) = W [u+0.5, v+0.5, 1] (camera
                                       projection's world_from_index[:-1, :], projector.py:803) */
    const double *source_world;     /* host [n_views][3]: source position in world (center_in_world) */
    const double *ijk_from_world;   /* host [n_views][n_volumes][3][4]: each volume's IJK_from_world */
    float *intensity;               /* device [n_views][H][W], keV per photon (required) */
    float *photon_prob;             /* device [n_views][H][W] (required) */
    float *area_density;            /* device [n_views][n_materials][H][W] in g/cm^2, or NULL */
    float *solid_angle;             /* device [n_views][H][W] pixel solid angles (sr), or NULL;
                                       project_kernel.cu:14-133 */
    /* launch shape of DRR_FLAG_PERSISTENT (0 = default; drr_autotune picks them per workload) */
    int32_t tile_warps_x;           /* 1, 2 or 4 warps across a tile of 4 warps (tiles 8x16, 16x8, 32x4) */
    int32_t blocks_per_sm;          /* resident 128-thread blocks per SM */
    int32_t items_per_grab;         /* tiles a block takes per atomic increment */
    /* additive meshes (drr_mesh_area_density): per view and mesh-material slot the path integral
       added to material mesh_material[slot]'s path length before the division by 10
       (project_kernel.cu:569-579); NULL for none */
    const float *mesh_area_density; /* device [n_views][n_mesh_slots][H][W], mm g/cm^3 */
    int32_t n_mesh_slots;
    const int32_t *mesh_material;   /* host [n_mesh_slots]: material index of each slot */
    /* subtractive meshes (drr_mesh_hits, n_views must be 1): samples inside any layer's surfaces add
       nothing, neither volume nor air (project_kernel.cu:498-521); NULL for none */
    const float *mesh_hit_alpha;    /* device [mesh_hit_layers][H][W][max_mesh_hits] */
    const int8_t *mesh_hit_facing;  /* device, same shape */
    int32_t mesh_hit_layers;
    int32_t max_mesh_hits;
} drr_project_args;

#define DRR_MAX_MESH_LAYERS 4

enum { DRR_MESH_ADDITIVE = 1, DRR_MESH_SUBTRACTIVE = 2 };

/* Triangles of the meshes of a projector. */
typedef struct {
    const float *triangles; /* device [n_triangles][3][3]: vertices in world coordinates (mm), wound so the
                               right-handed normal points out of the closed surface */
    const int32_t *slot;    /* device [n_triangles]: mesh-material slot in [0, n_slots) */
    const float *density;   /* device [n_triangles]: density of the triangle's mesh (g/cm^3) */
    const int32_t *layer;   /* device [n_triangles]: mesh layer in [0, n_layers), or NULL for all 0 */
    const uint8_t *mode;    /* device [n_triangles]: DRR_MESH_ADDITIVE | DRR_MESH_SUBTRACTIVE bits, or NULL
                               for all additive */
    int32_t n_triangles;
    int32_t n_slots;
    int32_t n_layers;       /* layers of the subtractive hit lists, [0, DRR_MAX_MESH_LAYERS] */
} drr_mesh_desc;

/* Subtractive hit lists of ONE view (the view's ray matrix and source as in drr_project_args): per
 * layer and pixel the distances along the pixel's centre ray at which it crosses the layer's
 * subtractive surfaces, sorted, with facing +1 entering and -1 leaving and 0 after the last (at most
 * max_hits, even, kept; further crossings are dropped). hit_alpha / hit_facing are device
 * [n_layers][H][W][max_hits]. Replaces the reference's depth-peeled hit textures and their clean-up
 * (projector.py:1124-1256, peel_postprocess_kernel.cu:15-235). */
drr_status drr_mesh_hits(const drr_mesh_desc *mesh, int32_t width, int32_t height, const double *world_from_index,
                         const double *source_world, int32_t max_hits, float *hit_alpha, int8_t *hit_facing,
                         void *stream);

/* Path integrals of additive meshes through every pixel of `n_views` views (the views' ray matrices
 * and sources as in drr_project_args), into `out` (device [n_views][n_slots][H][W], mm g/cm^3):
 * per slot max(sum of signed distance x density over the surfaces the pixel's centre ray crosses, 0)
 * where the crossings balance, else 0. With subtractive hit lists (one view only), the parts of a
 * layer-l additive mesh inside the consecutive hit pairs of every layer above l are removed, as the
 * reference's density_between pass does (shaders/density_between.frag, projector.py:1258-1300).
 * Replaces the reference's OpenGL density pass (pyrenderdrr/renderer.py, shaders/density.frag:9-13)
 * and its read-back (projector.py:1063-1088, 1302-1330); rasterised in CUDA with 1/256-pixel snapping
 * and a top-left rule, so shared edges count once. Triangles reaching behind the source are not
 * rasterised. */
drr_status drr_mesh_area_density(const drr_mesh_desc *mesh, int32_t width, int32_t height, int32_t n_views,
                                 const double *world_from_index, const double *source_world,
                                 const float *hit_alpha, const int8_t *hit_facing, int32_t max_hits, float *out,
                                 void *stream);

/* Render `args->n_views` views into the caller's device buffers, asynchronously on `stream`.
 * Replaces projector.py:709-800 and the projectKernel launch (project_kernel.cu:135-650).
 * Without DRR_FLAG_PERSISTENT every group of 32 views is one launch with the geometry in the
 * kernel parameters. With it, all views go into one persistent launch whose view records are
 * staged through library-owned pinned and device buffers (one staging per volume set: calls on
 * one volume set from several streams at once must be ordered by the caller). */
drr_status drr_project(drr_volset *set, const drr_tables *tables, const drr_project_args *args, void *stream);

/* A persistent projection captured in a CUDA graph (upload of the view records, reset of the work
 * counter, kernel), replayed by drr_graph_launch. The output pointers, volume set, tables, sizes
 * and launch shape of `args` are fixed at creation; the view geometry can be replaced between
 * replays with drr_graph_set_views (same number of views). No counterpart in the reference: this
 * replaces its serial loop over views (projector.py:679-685) for many views per call. */
typedef struct drr_graph drr_graph;
drr_status drr_graph_create(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                            drr_graph **out);
drr_status drr_graph_set_views(drr_graph *graph, const double *world_from_index, const double *source_world,
                               const double *ijk_from_world);
drr_status drr_graph_launch(drr_graph *graph, void *stream);
drr_status drr_graph_destroy(drr_graph *graph);

/* Launch-shape autotuner of the persistent projection: times candidate shapes on `args` (up to
 * `max_views` of its views; the outputs are overwritten) on `stream` and returns the fastest.
 * No counterpart in the reference. */
typedef struct {
    int32_t tile_warps_x;
    int32_t blocks_per_sm;
    int32_t items_per_grab;
    float ms_per_view;
} drr_tune_result;
drr_status drr_autotune(drr_volset *set, const drr_tables *tables, const drr_project_args *args, int32_t max_views,
                        void *stream, drr_tune_result *best);

/* Upstream gradients and gradient outputs of drr_project_adjoint. Device pointers. `struct_size`
 * must be sizeof(drr_adjoint_args), as for drr_project_args. */
typedef struct {
    uint32_t struct_size;           /* sizeof(drr_adjoint_args) */
    const float *area_density;      /* [n_views][n_materials][H][W]: drr_project's area_density for the
                                       same args, or NULL to recompute it (stream-ordered scratch) */
    const float *grad_intensity;    /* [n_views][H][W] dL/d(intensity), or NULL */
    const float *grad_photon_prob;  /* [n_views][H][W] dL/d(photon_prob), or NULL */
    const float *grad_area_density; /* [n_views][n_materials][H][W] dL/d(area_density), or NULL */
    float *grad_density;            /* [nk][nj][ni] dL/d(density), accumulated into; or NULL */
    float *grad_pose;               /* [n_views][6] dL/d(translation xyz, rotation vector xyz) of a rigid
                                       motion of the volume about `center` (world frame, at zero
                                       motion), accumulated into; or NULL */
    double center[3];               /* rotation centre, world */
} drr_adjoint_args;

/* Gradients of a loss through drr_project for one enabled volume without DRR_FLAG_ATTENUATE_OUTSIDE,
 * at most 32767 voxels per axis (else DRR_ERR_UNSUPPORTED). The density gradient is the exact
 * adjoint of the kernel's samples, with the texture unit's 8-bit corner weights; the pose gradient
 * differentiates the continuous trilinear interpolation of the same texels and labels, with the
 * march's sample positions held fixed. No counterpart in the reference (its projector is not
 * differentiable). */
drr_status drr_project_adjoint(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                               const drr_adjoint_args *adjoint, void *stream);

/* Detector noise of Projector(add_noise=True): replaces analytic_generators.add_noise
 * (deepdrr/projector/analytic_generators.py:10-18, called at projector.py:691-695). For `n_views`
 * [height][width] float32 images, lambda = photon_prob * photon_count (float32) and
 *   out = clip(intensity + convolve2d((Poisson(lambda) - lambda) * intensity / lambda, K, "same"), 0, 1e31)
 * with K the reference's 3x3 shot-noise kernel, zero fill at the borders, the arithmetic after the
 * variate in float64 and the result rounded to float32. The reference's electronic-noise term has
 * factor 0 and is not generated. Variates are Philox4x32-10 (key `seed`, counter = the pixel's flat
 * index view * H * W + row * W + column) through inversion (lambda < 10) or Hoermann's PTRS, so a
 * seed gives the same images on any launch shape. `out` must not alias the inputs; a pixel with
 * photon_prob 0 gives NaN in its 3x3 neighbourhood, as in the reference (0 / 0). */
drr_status drr_add_noise(const float *intensity, const float *photon_prob, float *out, int32_t n_views,
                         int32_t height, int32_t width, double photon_count, uint64_t seed, void *stream);

/* The variates drr_add_noise draws: out[i] = Poisson(lambda[i]) with counter i under key `seed`
 * (float32, exact below 2^24; NaN for a negative or non-finite lambda). */
drr_status drr_poisson_sample(const float *lambda, int64_t n, uint64_t seed, float *out, void *stream);

/* In-place negative-log transform of `n_views` float32 images of `pixels_per_view` pixels each,
 * on `stream`: per view x += min(x) + epsilon; x = -log(x); x = (x - min) / (max - min), and every
 * view becomes 0 if any view is constant. Replaces deepdrr/utils/image_utils.py:18-58 (`_neglog`,
 * applied by Projector.project at projector.py:700-702). Uses 12 bytes per view (plus 4) of
 * stream-ordered scratch (cudaMallocAsync). */
drr_status drr_neglog(float *images, int32_t n_views, int64_t pixels_per_view, float epsilon, void *stream);

/* drr_neglog for callers that cannot allocate device memory. This entry point has no counterpart
 * in the reference. Hosts that own the allocator and budget every byte up front, real-time loops
 * in which cudaMalloc or cudaFree would stall the device, and pipelines that record their work
 * into CUDA graphs while forbidding allocation calls all need a transform that allocates nothing.
 * It computes exactly what drr_neglog computes but keeps its scratch (3 words per view) in one
 * fixed device array inside the library, about 48 KiB that every GPU loading the library keeps until
 * the process exits; n_views above 4096 is rejected with DRR_ERR_UNSUPPORTED. The first call in a
 * CUDA context (on each device, and again after a cudaDeviceReset or under another driver context)
 * looks up that array's device address in the context and caches it: make that first call before
 * any stream capture. All calls share the array: calls whose work overlaps on the GPU, on any
 * streams, race and must be ordered by the caller. Each call resets the words it uses before
 * reading them. */
drr_status drr_neglog_noalloc(float *images, int32_t n_views, int64_t pixels_per_view, float epsilon, void *stream);

/* Collected energy of Projector(collected_energy=True): replaces Projector._calculate_collected_energy_per_pixel
 * (deepdrr/projector/projector.py:833-853). For `n_views` float32 views of `pixels_per_view` pixels
 *   out = intensity * solid_angle * photon_count / mean(solid_angle of the view) / pixel_area[view]
 * (keV per mm^2) in float32 operations in the reference's order; pixel_area (host, [n_views]) is the
 * reference's (SDD / fx) * (SDD / fy), rounded to float32 as numpy does for a float32 array. The mean
 * is the correctly rounded float32 mean of the view's solid angles (summed in float64). `out` may be
 * `intensity`. Uses 8 bytes per view of stream-ordered scratch (cudaMallocAsync). */
drr_status drr_collected_energy(const float *intensity, const float *solid_angle, float *out, int32_t n_views,
                                int64_t pixels_per_view, double photon_count, const double *pixel_area, void *stream);

/* In-place min(x, upper) over `n` floats: Projector(intensity_upper_bound=...), projector.py:697-698. */
drr_status drr_clip_upper(float *images, int64_t n, float upper, void *stream);

/* Human-readable description of the last error raised on this host thread ("" if none). */
const char *drr_last_error(void);

/* Library version string. */
const char *drr_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DRR_GB300_H */
