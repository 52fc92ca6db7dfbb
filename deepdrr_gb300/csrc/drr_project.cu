// drr_project.cu -- projection entry points of libdrr_gb300.so.
//
// Host-side replacement for deepdrr/projector/projector.py (deepdrr v1.2.2):
//   _update_object_locations  projector.py:802-831 -> pack_view()
//   _render_single            projector.py:709-800 -> drr_project()
// plus the persistent batched launch, its CUDA-graph capture and its launch-shape autotuner.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/drr_gb300.h"
#include "drr_adjoint.cuh"
#include "drr_forward.cuh"
#include "drr_internal.h"

using drr::cuda_fail;
using drr::fail;

namespace {

// _update_object_locations (projector.py:802-831): float64 host geometry cast to float32. The
// source position in IJK is computed in float64 in a fixed order, ((a0 s0 + a1 s1) + a2 s2) + a3.
template <int NV>
void pack_view(const double *world_from_index, const double *source_world, const double *ijk_from_world, int nvol,
               int view, drr::ViewRec<NV> &rec) {
    const double *W = world_from_index + (size_t)view * 9;
    for (int j = 0; j < 9; j++) rec.w[j] = (float)W[j];
    rec.pad = 0.0f;
    const double *src = source_world + (size_t)view * 3;
    for (int i = 0; i < NV; i++) {
        drr::VolPose &vp = rec.vol[i];
        if (i >= nvol) {
            std::memset(&vp, 0, sizeof(vp));
            continue;
        }
        const double *A = ijk_from_world + ((size_t)view * nvol + i) * 12;
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) vp.a[r * 3 + c] = (float)A[r * 4 + c];
            volatile double acc = A[r * 4 + 0] * src[0];
            acc = acc + A[r * 4 + 1] * src[1];
            acc = acc + A[r * 4 + 2] * src[2];
            acc = acc + A[r * 4 + 3];
            vp.s[r] = (float)acc;
        }
    }
}

int material_bucket(int m) {
    if (m <= 2) return 2;
    if (m <= 3) return 3;
    if (m <= 4) return 4;
    if (m <= 6) return 6;
    if (m <= 8) return 8;
    return 16;
}

template <int NV>
void fill_scene(drr::SceneParams<NV> &p, const drr_volset *set, const drr_tables *tab, const drr_project_args &a) {
    std::memset(&p, 0, sizeof(p));
    for (int i = 0; i < NV; i++) {
        const drr::Volume &v = set->vol[i];
        p.vol[i].density = v.density_tex;
        // code table addressed from the entry of base (0, 0, 0): two planes, two rows and two entries in
        const size_t origin = 2 * ((size_t)(v.ni + 2) * (size_t)(v.nj + 2) + (size_t)(v.ni + 2) + 1);
        p.vol[i].coded = v.coded ? v.coded + origin : nullptr;
        p.vol[i].gen_words = v.gen_words;
        p.vol[i].gen_start = v.gen_start;
        p.vol[i].n[0] = v.ni;
        p.vol[i].n[1] = v.nj;
        p.vol[i].n[2] = v.nk;
        p.vol[i].nm1[0] = (float)(v.ni - 1);
        p.vol[i].nm1[1] = (float)(v.nj - 1);
        p.vol[i].nm1[2] = (float)(v.nk - 1);
        p.vol[i].hi[0] = (float)(v.ni - 0.5);
        p.vol[i].hi[1] = (float)(v.nj - 0.5);
        p.vol[i].hi[2] = (float)(v.nk - 0.5);
        p.vol[i].row = v.ni + 2;
        p.vol[i].plane_bytes = (int32_t)(2 * (int64_t)(v.ni + 2) * (int64_t)(v.nj + 2));
        p.vol[i].priority = a.priority[i];
        p.vol[i].enabled = a.enabled[i] ? 1 : 0;
    }
    p.energies = tab->d_buf;
    p.pdf = tab->d_buf + tab->n_bins;
    p.mu = tab->d_buf + 2 * tab->n_bins;
    p.intensity = a.intensity;
    p.photon_prob = a.photon_prob;
    p.area_density = a.area_density;
    p.solid_angle = a.solid_angle;
    p.width = a.width;
    p.height = a.height;
    p.n_materials = set->n_materials;
    p.n_bins = tab->n_bins;
    p.step = a.step;
    p.max_ray_length = a.max_ray_length;
    p.attenuate = (a.flags & DRR_FLAG_ATTENUATE_OUTSIDE) ? 1 : 0;
    p.air_index = a.air_index;
    p.full_march = (a.flags & DRR_FLAG_FULL_MARCH) ? 1 : 0;
    p.mesh_ad = a.mesh_area_density;
    p.n_mesh = a.mesh_area_density ? a.n_mesh_slots : 0;
    for (int k = 0; k < p.n_mesh && k < drr::kMaxMeshSlots; k++) p.mesh_mat[k] = a.mesh_material[k];
    p.hit_alpha = a.mesh_hit_alpha;
    p.hit_facing = a.mesh_hit_facing;
    p.hit_layers = a.mesh_hit_alpha ? a.mesh_hit_layers : 0;
    p.max_hits = a.mesh_hit_alpha ? a.max_mesh_hits : 0;
}

template <int NV>
cudaError_t dispatch_plain(const drr::ForwardParams<NV> &p, int bucket, cudaStream_t s) {
    switch (bucket) {
        case 2: return drr::launch_forward<NV, 2>(p, s);
        case 3: return drr::launch_forward<NV, 3>(p, s);
        case 4: return drr::launch_forward<NV, 4>(p, s);
        case 6: return drr::launch_forward<NV, 6>(p, s);
        case 8: return drr::launch_forward<NV, 8>(p, s);
        default: return drr::launch_forward<NV, 16>(p, s);
    }
}

template <int NV>
cudaError_t dispatch_persistent(const drr::PersistentParams<NV> &p, int bucket, int grid, cudaStream_t s) {
    switch (bucket) {
        case 2: return drr::launch_persistent<NV, 2>(p, grid, s);
        case 3: return drr::launch_persistent<NV, 3>(p, grid, s);
        case 4: return drr::launch_persistent<NV, 4>(p, grid, s);
        case 6: return drr::launch_persistent<NV, 6>(p, grid, s);
        case 8: return drr::launch_persistent<NV, 8>(p, grid, s);
        default: return drr::launch_persistent<NV, 16>(p, grid, s);
    }
}

template <int NV>
int occupancy(int bucket) {
    switch (bucket) {
        case 2: return drr::persistent_occupancy<NV, 2>();
        case 3: return drr::persistent_occupancy<NV, 3>();
        case 4: return drr::persistent_occupancy<NV, 4>();
        case 6: return drr::persistent_occupancy<NV, 6>();
        case 8: return drr::persistent_occupancy<NV, 8>();
        default: return drr::persistent_occupancy<NV, 16>();
    }
}

template <int NV>
drr_status project_plain(drr_volset *set, const drr_tables *tab, const drr_project_args &a, cudaStream_t s) {
    drr::ForwardParams<NV> *pp = new (std::nothrow) drr::ForwardParams<NV>();
    if (!pp) return fail(DRR_ERR_OUT_OF_MEMORY, "drr_project: host allocation failed");
    drr::ForwardParams<NV> &p = *pp;
    fill_scene<NV>(p.s, set, tab, a);
    const int bucket = material_bucket(set->n_materials);
    drr_status st = DRR_OK;
    for (int v0 = 0; v0 < a.n_views; v0 += drr::kViewsPerLaunch) {
        const int nv = a.n_views - v0 < drr::kViewsPerLaunch ? a.n_views - v0 : drr::kViewsPerLaunch;
        p.view0 = v0;
        p.n_views = nv;
        for (int k = 0; k < nv; k++)
            pack_view<NV>(a.world_from_index, a.source_world, a.ijk_from_world, set->n_volumes, v0 + k, p.views[k]);
        cudaError_t e = dispatch_plain<NV>(p, bucket, s);
        if (e != cudaSuccess) {
            st = cuda_fail(e, "drr_project: kernel launch");
            break;
        }
    }
    delete pp;
    return st;
}

struct Shape {
    int warps_x, blocks_per_sm, grab;
};

template <int NV>
drr_status resolve_shape(const drr_volset *set, const drr_project_args &a, Shape *out) {
    const int bucket = material_bucket(set->n_materials);
    const int occ = occupancy<NV>(bucket);
    if (occ < 1) return fail(DRR_ERR_CUDA, "drr_project: occupancy query failed");
    Shape sh;
    sh.warps_x = a.tile_warps_x ? a.tile_warps_x : 2;
    sh.blocks_per_sm = a.blocks_per_sm ? a.blocks_per_sm : occ;
    sh.grab = a.items_per_grab ? a.items_per_grab : 1;
    if (sh.warps_x != 1 && sh.warps_x != 2 && sh.warps_x != 4)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: tile_warps_x must be 1, 2 or 4");
    if (sh.blocks_per_sm < 1 || sh.blocks_per_sm > 64 || sh.grab < 1 || sh.grab > 64)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: blocks_per_sm and items_per_grab must be in [1, 64]");
    *out = sh;
    return DRR_OK;
}

// Kernel parameters of a persistent launch whose view records are at `d_views`.
template <int NV>
drr_status persistent_params(const drr_volset *set, const drr_tables *tab, const drr_project_args &a,
                             const Shape &sh, const void *d_views, unsigned int *counter,
                             drr::PersistentParams<NV> *p) {
    fill_scene<NV>(p->s, set, tab, a);
    const int tile_w = 8 * sh.warps_x, tile_h = 4 * (4 / sh.warps_x);
    p->views = (const drr::ViewRec<NV> *)d_views;
    p->n_views = a.n_views;
    p->tiles_x = (a.width + tile_w - 1) / tile_w;
    p->tiles_y = (a.height + tile_h - 1) / tile_h;
    p->warps_x = sh.warps_x;
    p->items_per_grab = sh.grab;
    p->counter = counter;
    const double items = (double)p->tiles_x * p->tiles_y * a.n_views;
    if (items + (double)sh.grab * 65536.0 * 64.0 > 4294967295.0)
        return fail(DRR_ERR_UNSUPPORTED, "drr_project: too many (view, tile) items for one persistent launch");
    return DRR_OK;
}

template <int NV>
void pack_all(const drr_project_args &a, int nvol, void *host) {
    drr::ViewRec<NV> *rec = (drr::ViewRec<NV> *)host;
    for (int k = 0; k < a.n_views; k++) pack_view<NV>(a.world_from_index, a.source_world, a.ijk_from_world, nvol, k, rec[k]);
}

template <int NV>
drr_status project_persistent(drr_volset *set, const drr_tables *tab, const drr_project_args &a, cudaStream_t s) {
    Shape sh;
    drr_status st = resolve_shape<NV>(set, a, &sh);
    if (st != DRR_OK) return st;
    drr::Staging &stg = set->staging;
    const size_t bytes = (size_t)a.n_views * sizeof(drr::ViewRec<NV>);
    st = drr::ensure_staging(stg, bytes);
    if (st != DRR_OK) return st;
    if (stg.pending) cudaEventSynchronize(stg.uploaded);  // the previous upload still reads `host`
    pack_all<NV>(a, set->n_volumes, stg.host);
    drr::PersistentParams<NV> p;
    st = persistent_params<NV>(set, tab, a, sh, stg.device, stg.counter, &p);
    if (st != DRR_OK) return st;
    cudaError_t e = cudaMemcpyAsync(stg.device, stg.host, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(stg.uploaded, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(stg.counter, 0, sizeof(unsigned int), s);
    stg.pending = true;
    if (e != cudaSuccess) return cuda_fail(e, "drr_project: staging the view records");
    e = dispatch_persistent<NV>(p, material_bucket(set->n_materials), set->sm_count * sh.blocks_per_sm, s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_project: persistent kernel launch");
    return DRR_OK;
}

// The caller's struct must be this library's drr_project_args: checked before any other field is read.
drr_status check_struct_size(const drr_project_args *args) {
    if (!args) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL args");
    if (args->struct_size != sizeof(drr_project_args))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: args->struct_size is " + std::to_string(args->struct_size) +
                                                  ", this library's drr_project_args has " +
                                                  std::to_string(sizeof(drr_project_args)) + " bytes");
    return DRR_OK;
}

drr_status validate(const drr_volset *set, const drr_tables *tables, const drr_project_args *args) {
    const drr_status sz = check_struct_size(args);
    if (sz != DRR_OK) return sz;
    if (!set || !tables) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL handle");
    const drr_project_args &a = *args;
    if (a.width < 1 || a.height < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: empty detector");
    if ((int64_t)a.width * a.height > (int64_t)1 << 28)
        return fail(DRR_ERR_UNSUPPORTED, "drr_project: detector larger than 2^28 pixels");
    if (a.height > 65535 * drr::kTileH) return fail(DRR_ERR_UNSUPPORTED, "drr_project: detector too tall");
    if (a.n_views < 0) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: n_views < 0");
    if (!(a.step > 0.0f) || !std::isfinite(a.step))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: step must be a positive finite number");
    if (!a.priority || !a.enabled || !a.world_from_index || !a.source_world || !a.ijk_from_world)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL geometry pointer");
    if (!a.intensity || !a.photon_prob) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: NULL output pointer");
    if (tables->n_materials != set->n_materials)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: tables and volume set disagree on n_materials");
    for (int i = 0; i < set->n_volumes; i++)
        if (a.priority[i] < 0 || a.priority[i] >= set->n_volumes)
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: priority outside [0, n_volumes)");
    if ((a.flags & DRR_FLAG_ATTENUATE_OUTSIDE) && (a.air_index < 0 || a.air_index >= set->n_materials))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: air_index outside [0, n_materials)");
    if (a.mesh_hit_alpha) {
        if (!a.mesh_hit_facing || a.mesh_hit_layers < 1 || a.mesh_hit_layers > drr::kMaxMeshLayers ||
            a.max_mesh_hits < 2 || a.n_views > 1)
            return fail(DRR_ERR_INVALID_ARGUMENT,
                        "drr_project: subtractive hit lists need facings, 1-4 layers, max_mesh_hits >= 2 and one view");
    }
    if (a.mesh_area_density) {
        if (a.n_mesh_slots < 1 || a.n_mesh_slots > drr::kMaxMeshSlots || !a.mesh_material)
            return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: mesh slots outside [1, 16] or no slot materials");
        for (int k = 0; k < a.n_mesh_slots; k++)
            if (a.mesh_material[k] < 0 || a.mesh_material[k] >= set->n_materials)
                return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project: mesh slot material outside [0, n_materials)");
    }
    return DRR_OK;
}

template <template <int> class F, typename... Args>
drr_status by_volumes(int n_volumes, Args &&...args) {
    switch (n_volumes) {
        case 1: return F<1>::run(args...);
        case 2: return F<2>::run(args...);
        case 3: return F<3>::run(args...);
        default: return F<4>::run(args...);
    }
}

template <int NV>
struct ProjectOp {
    static drr_status run(drr_volset *set, const drr_tables *tab, const drr_project_args &a, cudaStream_t s) {
        return (a.flags & DRR_FLAG_PERSISTENT) ? project_persistent<NV>(set, tab, a, s) : project_plain<NV>(set, tab, a, s);
    }
};

}  // namespace

extern "C" drr_status drr_project(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                                  void *stream) {
    drr::set_last_error("");
    drr_status st = validate(set, tables, args);
    if (st != DRR_OK) return st;
    if (args->n_views == 0) return DRR_OK;
    return by_volumes<ProjectOp>(set->n_volumes, set, tables, *args, (cudaStream_t)stream);
}

// ---- CUDA graph of a persistent projection ------------------------------------------------------

struct drr_graph {
    drr_volset *set = nullptr;
    const drr_tables *tables = nullptr;
    drr_project_args args;
    std::vector<int32_t> priority, enabled;
    int n_volumes = 0;
    size_t record_bytes = 0;
    void *host = nullptr;    // pinned view records read by the graph's upload node
    void *device = nullptr;
    unsigned int *counter = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
    bool launched = false;
};

namespace {

void free_graph(drr_graph *g) {
    if (g->done) {
        if (g->launched) cudaEventSynchronize(g->done);
        cudaEventDestroy(g->done);
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->host) cudaFreeHost(g->host);
    if (g->device) cudaFree(g->device);
    if (g->counter) cudaFree(g->counter);
    delete g;
}

template <int NV>
struct GraphOp {
    static drr_status run(drr_graph *g) {
        const drr_project_args &a = g->args;
        Shape sh;
        drr_status st = resolve_shape<NV>(g->set, a, &sh);
        if (st != DRR_OK) return st;
        g->record_bytes = (size_t)a.n_views * sizeof(drr::ViewRec<NV>);
        cudaError_t e = cudaMallocHost(&g->host, g->record_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&g->device, g->record_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&g->counter, sizeof(unsigned int));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "drr_graph_create: buffers");
        pack_all<NV>(a, g->n_volumes, g->host);
        drr::PersistentParams<NV> p;
        st = persistent_params<NV>(g->set, g->tables, a, sh, g->device, g->counter, &p);
        if (st != DRR_OK) return st;
        cudaStream_t cs = nullptr;
        e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "drr_graph_create: capture stream");
        e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e1 = cudaMemcpyAsync(g->device, g->host, g->record_bytes, cudaMemcpyHostToDevice, cs);
            cudaError_t e2 = cudaMemsetAsync(g->counter, 0, sizeof(unsigned int), cs);
            cudaError_t e3 = dispatch_persistent<NV>(p, material_bucket(g->set->n_materials),
                                                     g->set->sm_count * sh.blocks_per_sm, cs);
            e = cudaStreamEndCapture(cs, &g->graph);
            if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3);
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess) return cuda_fail(e, "drr_graph_create: capture");
        return DRR_OK;
    }
};

template <int NV>
struct GraphViewsOp {
    static drr_status run(drr_graph *g) {
        pack_all<NV>(g->args, g->n_volumes, g->host);
        return DRR_OK;
    }
};

template <int NV>
struct OccupancyOp {
    static drr_status run(const drr_volset *set, int *occ) {
        *occ = occupancy<NV>(material_bucket(set->n_materials));
        return *occ > 0 ? DRR_OK : fail(DRR_ERR_CUDA, "drr_autotune: occupancy query failed");
    }
};

}  // namespace

extern "C" drr_status drr_graph_create(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                                       drr_graph **out) {
    drr::set_last_error("");
    if (!out) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_graph_create: out is NULL");
    *out = nullptr;
    drr_status st = validate(set, tables, args);
    if (st != DRR_OK) return st;
    if (args->n_views < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_graph_create: no views");
    drr_graph *g = new (std::nothrow) drr_graph();
    if (!g) return fail(DRR_ERR_OUT_OF_MEMORY, "drr_graph_create: host allocation failed");
    g->set = set;
    g->tables = tables;
    g->args = *args;
    g->n_volumes = set->n_volumes;
    g->priority.assign(args->priority, args->priority + set->n_volumes);
    g->enabled.assign(args->enabled, args->enabled + set->n_volumes);
    g->args.priority = g->priority.data();
    g->args.enabled = g->enabled.data();
    g->args.flags |= DRR_FLAG_PERSISTENT;
    st = by_volumes<GraphOp>(set->n_volumes, g);
    if (st != DRR_OK) {
        free_graph(g);
        return st;
    }
    g->args.mesh_material = nullptr;     // copied into the captured kernel parameters
    g->args.world_from_index = nullptr;  // the caller's geometry arrays are not kept
    g->args.source_world = nullptr;
    g->args.ijk_from_world = nullptr;
    *out = g;
    return DRR_OK;
}

extern "C" drr_status drr_graph_set_views(drr_graph *g, const double *world_from_index, const double *source_world,
                                          const double *ijk_from_world) {
    drr::set_last_error("");
    if (!g || !world_from_index || !source_world || !ijk_from_world)
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_graph_set_views: NULL argument");
    if (g->launched) {
        cudaError_t e = cudaEventSynchronize(g->done);  // the last replay's upload still reads `host`
        if (e != cudaSuccess) return cuda_fail(e, "drr_graph_set_views: waiting for the last replay");
    }
    g->args.world_from_index = world_from_index;
    g->args.source_world = source_world;
    g->args.ijk_from_world = ijk_from_world;
    drr_status st = by_volumes<GraphViewsOp>(g->n_volumes, g);
    g->args.world_from_index = g->args.source_world = g->args.ijk_from_world = nullptr;
    return st;
}

extern "C" drr_status drr_graph_launch(drr_graph *g, void *stream) {
    drr::set_last_error("");
    if (!g) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_graph_launch: NULL graph");
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaEventRecord(g->done, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "drr_graph_launch");
    g->launched = true;
    return DRR_OK;
}

extern "C" drr_status drr_graph_destroy(drr_graph *g) {
    drr::set_last_error("");
    if (g) free_graph(g);
    return DRR_OK;
}

// ---- launch-shape autotuner ----------------------------------------------------------------------

extern "C" drr_status drr_autotune(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                                   int32_t max_views, void *stream, drr_tune_result *best) {
    drr::set_last_error("");
    drr_status st = validate(set, tables, args);
    if (st != DRR_OK) return st;
    if (!best) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_autotune: best is NULL");
    if (args->n_views < 1) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_autotune: no views");
    cudaStream_t s = (cudaStream_t)stream;
    drr_project_args a = *args;
    a.flags |= DRR_FLAG_PERSISTENT;
    if (max_views > 0 && a.n_views > max_views) a.n_views = max_views;
    // occupancy of this (volumes, materials) kernel bounds the resident-block candidates
    a.tile_warps_x = 2;
    a.blocks_per_sm = 0;
    a.items_per_grab = 1;
    int occ = 0;
    st = by_volumes<OccupancyOp>(set->n_volumes, set, &occ);
    if (st != DRR_OK) return st;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(DRR_ERR_CUDA, "drr_autotune: cudaEventCreate failed");
    const int wxs[3] = {1, 2, 4};
    const int bps[3] = {occ > 1 ? occ / 2 : 1, occ, 2 * occ};
    const int grabs[2] = {1, 4};
    drr_tune_result r = {0, 0, 0, 1e30f};
    st = drr_project(set, tables, &a, stream);  // warm-up with the default shape
    for (int i = 0; i < 3 && st == DRR_OK; i++)
        for (int j = 0; j < 3 && st == DRR_OK; j++)
            for (int k = 0; k < 2 && st == DRR_OK; k++) {
                a.tile_warps_x = wxs[i];
                a.blocks_per_sm = bps[j];
                a.items_per_grab = grabs[k];
                cudaEventRecord(e0, s);
                st = drr_project(set, tables, &a, stream);
                cudaEventRecord(e1, s);
                if (st != DRR_OK) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    st = fail(DRR_ERR_CUDA, "drr_autotune: timing failed");
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= (float)a.n_views;
                if (ms < r.ms_per_view) r = {wxs[i], bps[j], grabs[k], ms};
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != DRR_OK) return st;
    *best = r;
    return DRR_OK;
}

// ---- adjoint (density and pose gradients) --------------------------------------------------------

namespace {

cudaError_t dispatch_adjoint(const drr::AdjointParams &p, int bucket, cudaStream_t s) {
    switch (bucket) {
        case 2: return drr::launch_adjoint<2>(p, s);
        case 3: return drr::launch_adjoint<3>(p, s);
        case 4: return drr::launch_adjoint<4>(p, s);
        case 6: return drr::launch_adjoint<6>(p, s);
        case 8: return drr::launch_adjoint<8>(p, s);
        default: return drr::launch_adjoint<16>(p, s);
    }
}

drr_status ensure_point_texture(drr::Volume &v) {
    if (v.density_point) return DRR_OK;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = v.density_array;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaError_t e = cudaCreateTextureObject(&v.density_point, &rd, &td, nullptr);
    if (e != cudaSuccess) {
        v.density_point = 0;
        return cuda_fail(e, "drr_project_adjoint: point texture");
    }
    return DRR_OK;
}

}  // namespace

extern "C" drr_status drr_project_adjoint(drr_volset *set, const drr_tables *tables, const drr_project_args *args,
                                          const drr_adjoint_args *adj, void *stream) {
    drr::set_last_error("");
    const drr_status sz = check_struct_size(args);
    if (sz != DRR_OK) return sz;
    if (!adj) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project_adjoint: NULL adjoint args");
    if (adj->struct_size != sizeof(drr_adjoint_args))
        return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project_adjoint: adj->struct_size is " +
                                                  std::to_string(adj->struct_size) + ", this library's drr_adjoint_args has " +
                                                  std::to_string(sizeof(drr_adjoint_args)) + " bytes");
    if (!set || !tables) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project_adjoint: NULL argument");
    if (set->n_volumes != 1) return fail(DRR_ERR_UNSUPPORTED, "drr_project_adjoint: one volume only");
    if (args->flags & DRR_FLAG_ATTENUATE_OUTSIDE)
        return fail(DRR_ERR_UNSUPPORTED, "drr_project_adjoint: DRR_FLAG_ATTENUATE_OUTSIDE is not differentiated");
    // validate() wants the forward's outputs; the adjoint reads none of them
    drr_project_args a = *args;
    float dummy = 0.0f;
    a.intensity = a.photon_prob = &dummy;
    drr_status st = validate(set, tables, &a);
    if (st != DRR_OK) return st;
    if (!args->enabled[0]) return fail(DRR_ERR_INVALID_ARGUMENT, "drr_project_adjoint: the volume is disabled");
    {
        const drr::Volume &v = set->vol[0];
        if (v.ni > 32767 || v.nj > 32767 || v.nk > 32767)
            return fail(DRR_ERR_UNSUPPORTED, "drr_project_adjoint: volumes above 32767 voxels per axis");
    }
    if (args->n_views == 0 || (!adj->grad_density && !adj->grad_pose)) return DRR_OK;
    cudaStream_t s = (cudaStream_t)stream;
    st = ensure_point_texture(set->vol[0]);
    if (st != DRR_OK) return st;

    const int n = args->n_views, M = set->n_materials;
    const size_t plane = (size_t)args->width * args->height;
    std::vector<drr::AdjointView> views((size_t)n);
    for (int k = 0; k < n; k++) {
        pack_view<1>(args->world_from_index, args->source_world, args->ijk_from_world, 1, k, views[k].v);
        for (int c = 0; c < 3; c++) views[k].source_world[c] = (float)args->source_world[(size_t)k * 3 + c];
        views[k].pad = 0.0f;
    }
    void *d_views = nullptr;
    float *scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&d_views, views.size() * sizeof(drr::AdjointView), s);
    if (e != cudaSuccess) return cuda_fail(e, "drr_project_adjoint: cudaMallocAsync");
    e = cudaMemcpyAsync(d_views, views.data(), views.size() * sizeof(drr::AdjointView), cudaMemcpyHostToDevice, s);
    const float *ad = adj->area_density;
    if (e == cudaSuccess && ad == nullptr) {
        // recompute the forward's area densities into stream-ordered scratch
        const size_t floats = (size_t)n * plane * (2 + (size_t)M);
        e = cudaMallocAsync((void **)&scratch, floats * sizeof(float), s);
        if (e == cudaSuccess) {
            drr_project_args f = *args;
            f.flags &= ~(uint32_t)DRR_FLAG_PERSISTENT;
            f.intensity = scratch;
            f.photon_prob = scratch + (size_t)n * plane;
            f.area_density = scratch + 2 * (size_t)n * plane;
            f.solid_angle = nullptr;
            st = project_plain<1>(set, tables, f, s);
            ad = f.area_density;
        }
    }
    if (e == cudaSuccess && st == DRR_OK) {
        drr::AdjointParams p;
        std::memset(&p, 0, sizeof(p));
        fill_scene<1>(p.s, set, tables, a);
        p.s.intensity = p.s.photon_prob = nullptr;
        p.s.area_density = p.s.solid_angle = nullptr;
        p.density_point = set->vol[0].density_point;
        for (int c = 0; c < 3; c++) p.center[c] = (float)adj->center[c];
        const int bucket = material_bucket(M);
        for (int v0 = 0; v0 < n && e == cudaSuccess; v0 += 65535) {
            const int nv = n - v0 < 65535 ? n - v0 : 65535;
            p.views = (const drr::AdjointView *)d_views + v0;
            p.n_views = nv;
            p.area_density = ad + (size_t)v0 * M * plane;
            p.grad_intensity = adj->grad_intensity ? adj->grad_intensity + (size_t)v0 * plane : nullptr;
            p.grad_photon_prob = adj->grad_photon_prob ? adj->grad_photon_prob + (size_t)v0 * plane : nullptr;
            p.grad_area_density = adj->grad_area_density ? adj->grad_area_density + (size_t)v0 * M * plane : nullptr;
            p.grad_density = adj->grad_density;
            p.grad_pose = adj->grad_pose ? adj->grad_pose + (size_t)v0 * 6 : nullptr;
            e = dispatch_adjoint(p, bucket, s);
        }
    }
    if (scratch) cudaFreeAsync(scratch, s);
    cudaFreeAsync(d_views, s);
    if (st != DRR_OK) return st;
    if (e != cudaSuccess) return cuda_fail(e, "drr_project_adjoint");
    return DRR_OK;
}
