// drr_internal.h -- library-internal definitions shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/drr_gb300.h"

namespace drr {

void set_last_error(const std::string &msg);
drr_status fail(drr_status s, const std::string &msg);
drr_status cuda_fail(cudaError_t e, const char *what);

struct Volume {
    cudaArray_t density_array = nullptr;
    cudaTextureObject_t density_tex = 0;
    cudaTextureObject_t density_point = 0;  // point-filtered view of density_array (made by the adjoint)
    uint16_t *coded = nullptr;   // [(nk+2)][(nj+2)][(ni+2)] codes of the 2x2x2 label neighbourhoods
                                 // (A, B, corners labelled B; see pack_labels_kernel)
    uint32_t *gen_words = nullptr;  // packed labels of the neighbourhoods of three or more labels, numbered
    uint32_t *gen_start = nullptr;  // per segment of a code-table row (first index of each segment)
    int ni = 0, nj = 0, nk = 0;
    int density_type = DRR_DENSITY_F32;
};

// Staging of per-view records for persistent launches: pinned host memory, its device copy and
// the work counter. One set per volume set (calls on one volume set from several streams at once
// must be ordered by the caller).
struct Staging {
    void *host = nullptr;    // pinned
    void *device = nullptr;
    size_t capacity = 0;     // bytes of each buffer
    unsigned int *counter = nullptr;
    cudaEvent_t uploaded = nullptr;  // recorded after the last upload from `host`
    bool pending = false;
};

void free_staging(Staging &st);
drr_status ensure_staging(Staging &st, size_t bytes);

}  // namespace drr

struct drr_volset {
    int n_volumes = 0;
    int n_materials = 0;
    drr::Volume vol[DRR_MAX_VOLUMES];
    drr::Staging staging;
    int sm_count = 0;
};

struct drr_tables {
    int n_bins = 0;
    int n_materials = 0;
    float *d_buf = nullptr;  // energies [n_bins] | pdf [n_bins] | mu [n_bins][n_materials]
};
