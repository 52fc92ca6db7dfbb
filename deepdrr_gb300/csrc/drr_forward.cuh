// drr_forward.cuh -- forward DRR kernel (one thread per detector ray), sm_103a.
//
// Restates projectKernel of deepdrr/projector/project_kernel.cu:135-650 (deepdrr v1.2.2) with the
// same float32 arithmetic, operation by operation, so that results match the reference kernel:
//   * ray setup and normalisation                       project_kernel.cu:218-234
//   * per-volume slab test in IJK, boxes [-0.5, n-0.5]  project_kernel.cu:265-323
//   * num_steps = ceil((maxAlpha - minAlpha) / step)    project_kernel.cu:334
//   * float32 `alpha += step`, sample p = s + alpha r - 1 (the -1 voxel offset of both fields)
//                                                       project_kernel.cu:398-404, 552
//   * labels of the 2x2x2 neighbourhood re-read on voxel change, one cache shared by all volumes
//                                                       project_kernel.cu:394-431
//   * trilinear label fractions, priority resolution, trapezoid half weights, hardware-filtered
//     density, per-material accumulation                project_kernel.cu:433-551
//   * air tails, * step, / 10 (mm -> cm)                project_kernel.cu:358-361, 557-584
//   * polychromatic Beer-Lambert                        project_kernel.cu:637-646
// Every multiply-add is an explicit __fmaf_rn / __fmul_rn / __fadd_rn, grouped exactly as nvcc
// contracts the reference's expressions (a*b + c*d + e -> fma(a, b, c*d) + e; a*b + c*d + e*f ->
// fma(e, f, fma(a, b, c*d))), so sample positions are bit-identical to the reference kernel's.
//
// Differences from the reference, none of which changes a result:
//   * per-volume state lives in registers (NV, M are template parameters) instead of the
//     reference's 528-byte local-memory stack frame;
//   * the eight labels of a 2x2x2 neighbourhood come from one 16-bit load of a precomputed code
//     table (the neighbourhood's two labels and which corners hold the second, clamp addressing
//     folded in) instead of eight point-filtered texture fetches; the rare neighbourhoods with three
//     or more labels read their eight bytes from a copy of the label volume (fetch_label_word
//     explains why this reads exactly the reference's texels);
//   * steps before the first volume interval opens do no sampling (their float32 alpha sequence is
//     still accumulated step by step, so every later sample position is bit-identical), and the
//     march stops once alpha has passed the last interval. With more than one volume the last
//     skipped step is replayed in full so the shared label cache enters the first live step in the
//     reference's state. DRR_FLAG_FULL_MARCH disables both shortcuts;
//   * a neighbourhood whose eight labels agree adds to one material only (the reference adds
//     w * 0 = +0.0f to the others, which leaves them unchanged); its running sum is kept in a
//     register and written back when the material changes, which keeps the exact sequence of
//     float32 additions of every material;
//   * the reference's "all label weights zero" skip (project_kernel.cu:476-486) can never fire:
//     the eight trilinear weights are non-negative and one of them is at least 1/8;
//   * disabled volumes are ignored (the reference samples them with uninitialised directions);
//     the label cache starts empty where the reference leaves it uninitialised.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "drr_alpha.h"
#include "drr_coincide.h"

namespace drr {

constexpr int kViewsPerLaunch = 32;
constexpr int kMaxMeshSlots = 16;
constexpr int kMaxMeshLayers = 4;
constexpr int kBlockThreads = 128;  // 4 warps; each warp covers an 8 x 4 pixel tile
constexpr int kTileW = 16;          // block tile: 16 x 8 pixels
constexpr int kTileH = 8;
constexpr double kAirDensity = 0.1129;  // project_kernel.cu:5-7 (a double literal)
constexpr int kMaxSteps = 1 << 26;      // longest march per ray; longer rays are reported as NaN

struct VolConst {
    cudaTextureObject_t density;  // linear filter, clamp, unnormalised coordinates
    const uint16_t *coded;        // label codes [(nk+2)][(nj+2)][(ni+2)] (pack_labels_kernel), at the entry of
                                  // base (0, 0, 0): bases run from -2 to n - 1 on each axis
    const uint32_t *gen_words;    // packed labels of the neighbourhoods of three or more labels, numbered
    const uint32_t *gen_start;    // per row segment of the code table (general_label_word)
    int32_t n[3];                 // ni, nj, nk
    float hi[3];                  // n - 0.5 per axis (projector.py:1626-1634)
    float nm1[3];                 // n - 1 per axis
    int32_t priority;
    int32_t enabled;
    int32_t row;          // code-table entries per row: n[0] + 2
    int32_t plane_bytes;  // code-table bytes per plane: 2 (n[0] + 2)(n[1] + 2), below 2^31 because
                          // volumes are at most 16384 texels per axis (drr_volset_create)
};

struct VolPose {
    float a[9];  // 3x3 part of IJK_from_world (row-major), float32 as the reference host casts it
    float s[3];  // source position in IJK, float64 product cast to float32 (projector.py:812-820)
};

template <int NV>
struct ViewRec {
    float w[9];  // world_from_index[:-1, :] in float32 (projector.py:803)
    float pad;
    VolPose vol[NV];
};

// Everything a ray needs except its view.
template <int NV>
struct SceneParams {
    VolConst vol[NV];
    const float *energies;  // [n_bins] keV
    const float *pdf;       // [n_bins]
    const float *mu;        // [n_bins][n_materials]
    float *intensity;       // [views][H][W]
    float *photon_prob;     // [views][H][W]
    float *area_density;    // [views][n_materials][H][W] or null
    float *solid_angle;     // [views][H][W] or null
    int32_t width, height, n_materials, n_bins;
    float step, max_ray_length;
    int32_t attenuate, air_index;
    int32_t full_march;
    const float *mesh_ad;                 // [views][n_mesh][H][W] additive mesh integrals (mm g/cm^3) or null
    int32_t n_mesh;
    int32_t mesh_mat[kMaxMeshSlots];      // material of each mesh slot
    const float *hit_alpha;               // [hit_layers][H][W][max_hits] subtractive crossings (one view) or null
    const int8_t *hit_facing;
    int32_t hit_layers, max_hits;
};

// One launch of the plain kernel: up to kViewsPerLaunch views in the kernel parameters, one block
// per 16 x 8 pixel tile, blockIdx.z = view.
template <int NV>
struct ForwardParams {
    SceneParams<NV> s;
    int32_t view0;    // output index of views[0]
    int32_t n_views;  // views in this launch
    ViewRec<NV> views[kViewsPerLaunch];
};

// One launch of the persistent kernel: any number of views in device memory; resident blocks take
// (view, tile) work items from an atomic counter until none are left.
template <int NV>
struct PersistentParams {
    SceneParams<NV> s;
    const ViewRec<NV> *views;  // device [n_views]
    int32_t n_views;
    int32_t tiles_x, tiles_y;  // tiles per view
    int32_t warps_x;           // 1, 2 or 4 warps across a tile; a tile is (8 warps_x) x (16 / warps_x) pixels
    int32_t items_per_grab;    // tiles taken per counter increment
    unsigned int *counter;     // zero at launch
};

// ---- float32 groupings of the reference's dot products (see the file comment) ----------------
__device__ __forceinline__ float ray_component(float u, float a, float v, float b, float c) {
    return __fadd_rn(__fmaf_rn(u, a, __fmul_rn(v, b)), c);  // u*a + v*b + c
}
__device__ __forceinline__ float dot3(float a0, float x, float a1, float y, float a2, float z) {
    return __fmaf_rn(a2, z, __fmaf_rn(a0, x, __fmul_rn(a1, y)));  // a0*x + a1*y + a2*z
}

// Pixel solid angle from two tetrahedra, project_kernel.cu:14-133 (Van Oosterom-Strackee formula).
__device__ __forceinline__ float pixel_solid_angle(const float *w, int udx, int vdx) {
    float cx[4], cy[4], cz[4], cm[4];
    const float cu_off[4] = {0.f, 1.f, 1.f, 0.f};
    const float cv_off[4] = {0.f, 0.f, 1.f, 1.f};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        float cu = (float)udx + cu_off[c];
        float cv = (float)vdx + cv_off[c];
        cx[c] = ray_component(cu, w[0], cv, w[1], w[2]);
        cy[c] = ray_component(cu, w[3], cv, w[4], w[5]);
        cz[c] = ray_component(cu, w[6], cv, w[7], w[8]);
        cm[c] = __fsqrt_rn(dot3(cx[c], cx[c], cy[c], cy[c], cz[c], cz[c]));
    }
    const float kx = __fmaf_rn(cy[0], cz[2], -__fmul_rn(cz[0], cy[2]));
    const float ky = __fmaf_rn(cz[0], cx[2], -__fmul_rn(cx[0], cz[2]));
    const float kz = __fmaf_rn(cx[0], cy[2], -__fmul_rn(cy[0], cx[2]));
    const float d01 = dot3(cx[0], cx[1], cy[0], cy[1], cz[0], cz[1]);
    const float d02 = dot3(cx[0], cx[2], cy[0], cy[2], cz[0], cz[2]);
    const float d03 = dot3(cx[0], cx[3], cy[0], cy[3], cz[0], cz[3]);
    const float d12 = dot3(cx[1], cx[2], cy[1], cy[2], cz[1], cz[2]);
    const float d23 = dot3(cx[2], cx[3], cy[2], cy[3], cz[2], cz[3]);
    const float n012 = fabsf(dot3(cx[1], kx, cy[1], ky, cz[1], kz));
    const float n023 = fabsf(dot3(cx[3], kx, cy[3], ky, cz[3], kz));
    const float den012 = __fmaf_rn(d12, cm[0], __fmaf_rn(d02, cm[1],
                         __fmaf_rn(__fmul_rn(cm[0], cm[1]), cm[2], __fmul_rn(d01, cm[2]))));
    const float den023 = __fmaf_rn(d23, cm[0], __fmaf_rn(d03, cm[2],
                         __fmaf_rn(__fmul_rn(cm[0], cm[2]), cm[3], __fmul_rn(d02, cm[3]))));
    float sa012 = 2.f * atan2f(n012, den012);
    if (sa012 < 0.0f) sa012 += 3.14159265358979f;
    float sa023 = 2.f * atan2f(n023, den023);
    if (sa023 < 0.0f) sa023 += 3.14159265358979f;
    return sa012 + sa023;
}

// Paired float32 arithmetic: sm_103a's f32x2 instructions apply the scalar operation to two
// independent lanes in one instruction, each lane rounded to nearest exactly as __fmaf_rn /
// __fadd_rn / __fsub_rn / __fmul_rn round it (no flush of subnormals), so pairing the x and y halves
// of the march's vector arithmetic changes no result and saves an instruction per pair.
__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};"
        "\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tadd.rn.f32x2 rd, ra, rb;"
        "\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tsub.rn.f32x2 rd, ra, rb;"
        "\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

__device__ __forceinline__ float add_air(float x) {
    // area_density[AIR_INDEX] += AIR_DENSITY: a float32 accumulator plus a double literal
    return (float)((double)x + kAirDensity);
}

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// The eight labels the reference fetches at p + (dx, dy, dz) (point filter: texel clamp(floor)),
// with (bx, by, bz) = floor(p) and corner c = dx | dy << 1 | dz << 2.
// The reference's +1 corners read texel floor(p (+) 1) in float32; that always equals floor(p) + 1
// here because p = F (-) 1 with F = fma(alpha, r, s) a float: for |p| <= 2, p (+) 1 is exact
// (Sterbenz), and above that 1 is a multiple of ulp(p) (up to |p| = 2^24, far outside any volume,
// where both corners clamp to the same texel anyway). So the neighbourhood is a function of the
// base alone, precomputed per base b in [-2, n-1]^3 (pack_labels_kernel) as a 16-bit code:
//   bits 0-3   A, corner 0's label
//   bits 4-7   B, the other label of a two-label neighbourhood (A when there is none)
//   bits 9-15  the corners 1-7 labelled B (bit 8 + c for corner c)
//   bit 8      set for a neighbourhood of three or more labels (corner 0 is A by definition, so
//              this bit is otherwise always clear); its labels are then read from the volume.
// So a neighbourhood is uniform when code >> 8 == 0.
constexpr uint32_t kCodeGeneral = 0x100u;

// Entry of base (i, j, k), -2 <= i <= n[0] - 1 etc., of a code table [(n[2]+2)][(n[1]+2)][(n[0]+2)]
// given at the entry of base (0, 0, 0): the plane by one widening 32 x 32 -> 64-bit multiply, the
// offset inside it in 32-bit arithmetic (|offset| < (n[0]+2)(n[1]+2) <= 16386^2). This is the address
// of entry ((k+2)(n[1]+2) + j+2)(n[0]+2) + i+2 of the table's start, computed in 64 bits.
// Base -2 holds the same neighbourhood as base -1 (on that axis both corners clamp to texel 0); the
// extra layer lets marches whose bases provably stay in [-2, n-1] skip the clamps
// (fetch_label_code_direct).
__device__ __forceinline__ uint32_t label_entry(const uint16_t *origin, const VolConst &V, int i, int j, int k) {
    const char *plane = reinterpret_cast<const char *>(origin) + (long long)k * V.plane_bytes;
    return (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(plane) + (j * V.row + i));
}

// The code of base clamp(b, -1, n-1) (bases outside behave like the clamped one).
__device__ __forceinline__ uint32_t fetch_label_code(const VolConst &V, float bx, float by, float bz) {
    const int i = (int)fminf(fmaxf(bx, -1.0f), V.nm1[0]);
    const int j = (int)fminf(fmaxf(by, -1.0f), V.nm1[1]);
    const int k = (int)fminf(fmaxf(bz, -1.0f), V.nm1[2]);
    return label_entry(V.coded, V, i, j, k);
}

// The code of base b read without clamps: only for bases known to lie in [-2, n-1] on every axis,
// where the table has an entry equal to the clamped base's (see direct_bases).
__device__ __forceinline__ uint32_t fetch_label_code_direct(const VolConst &V, float bx, float by, float bz) {
    return label_entry(V.coded, V, (int)bx, (int)by, (int)bz);
}

// Whether a march may read its label codes without clamps. Its samples' positions
// fl(fl(fma(alpha, r, s)) - 1) and their floors are monotone in alpha on each axis (every operation
// is a monotone rounding), so every base it meets lies between the bases of its first and its last
// position (b0 and b1 here; the last is the look-ahead one step past its last sample, whose code
// the march also loads). Written as comparisons so that a NaN fails.
__device__ __forceinline__ bool direct_bases(const VolConst &V, float2 b0xy, float b0z, float2 b1xy, float b1z) {
    return b0xy.x >= -2.0f && b1xy.x >= -2.0f && b0xy.x <= V.nm1[0] && b1xy.x <= V.nm1[0] &&
           b0xy.y >= -2.0f && b1xy.y >= -2.0f && b0xy.y <= V.nm1[1] && b1xy.y <= V.nm1[1] &&
           b0z >= -2.0f && b1z >= -2.0f && b0z <= V.nm1[2] && b1z <= V.nm1[2];
}

// Neighbourhoods of three or more labels are numbered within segments of kGeneralSegment bases of
// a code-table row, so that a number fits the 11 bits a code of such a neighbourhood leaves free.
constexpr int kGeneralSegment = 2048;
__host__ __device__ __forceinline__ unsigned general_segments_per_row(int ni) {
    return (unsigned)(ni + 2 + kGeneralSegment - 1) / (unsigned)kGeneralSegment;
}

// The packed word of a neighbourhood of three or more labels, 4 bits per corner (corner c at bits
// 4c..4c+3: the eight texels the reference fetches with point filtering and clamp addressing,
// projector.py:1500-1519, at b + d + 0.5, whose texel is clamp(b + d, 0, n - 1)), whose code `code`
// was read at base (bx, by, bz), clamped to the table or not. The code carries the neighbourhood's
// number in its row segment (bits 4-7 and 9-15; drr_volset_create numbers them), so the word is
// two loads: the segment's first index and the word. The table's rows and plane of bases -2 are
// copies of those of -1, numbers included, so j and k are clamped to [-1, n - 1] here, and i only
// chooses the segment, which bases -2 and -1 share.
__device__ __forceinline__ uint32_t general_label_word(const VolConst &V, uint32_t code, float bx, float by, float bz) {
    const int i = (int)fminf(fmaxf(bx, -1.0f), V.nm1[0]);
    const int j = (int)fminf(fmaxf(by, -1.0f), V.nm1[1]);
    const int k = (int)fminf(fmaxf(bz, -1.0f), V.nm1[2]);
    const unsigned seg = ((unsigned)(k + 2) * (unsigned)(V.n[1] + 2) + (unsigned)(j + 2)) * general_segments_per_row(V.n[0]) +
                         (unsigned)(i + 2) / (unsigned)kGeneralSegment;
    const uint32_t number = ((code >> 4) & 15u) | ((code >> 9) << 4);
    return __ldg(V.gen_words + __ldg(V.gen_start + seg) + number);
}

// The packed word of a neighbourhood from its code, 4 bits per corner; (bx, by, bz) is the base the
// code belongs to. Codes of one or two labels expand arithmetically: the mask's bit c moves to bit
// 4c, and the corners it marks take B instead of A; three or more labels come from general_label_word.
__device__ __forceinline__ uint32_t code_word(const VolConst &V, uint32_t code, float bx, float by, float bz) {
    if (code & kCodeGeneral) return general_label_word(V, code, bx, by, bz);
    const uint32_t A = code & 15u, B = (code >> 4) & 15u;
    uint32_t m = code >> 8;                    // bit c: corner c holds B
    m = (m | (m << 12)) & 0x000F000Fu;         // spread bit c to bit 4c
    m = (m | (m << 6)) & 0x03030303u;
    m = (m | (m << 3)) & 0x11111111u;
    return (A * 0x11111111u) ^ ((A ^ B) * m);
}

__device__ __forceinline__ uint32_t fetch_label_word(const VolConst &V, float bx, float by, float bz) {
    const float cx = fminf(fmaxf(bx, -1.0f), V.nm1[0]);
    const float cy = fminf(fmaxf(by, -1.0f), V.nm1[1]);
    const float cz = fminf(fmaxf(bz, -1.0f), V.nm1[2]);
    return code_word(V, label_entry(V.coded, V, (int)cx, (int)cy, (int)cz), cx, cy, cz);
}

__device__ __forceinline__ bool uniform_word(uint32_t w) { return w == (w & 15u) * 0x11111111u; }

// Trilinear label weights (project_kernel.cu:441-448): corner c = dx | dy << 1 | dz << 2 has
// weight xy[c & 3] * z[c >> 2], with xy the four products (1-fx|fx)(1-fy|fy) rounded first.
// The reference adds each corner weight into seg[label] as seg = fma(xy, z, seg) (nvcc contracts
// the product into the accumulation), which is what uniform_sum and label_fractions do.
struct CornerWeights {
    float xy[4];
    float z[2];
};
__device__ __forceinline__ CornerWeights corner_weights(float fx, float fy, float fz) {
    const float gx = __fsub_rn(1.0f, fx), gy = __fsub_rn(1.0f, fy), gz = __fsub_rn(1.0f, fz);
    CornerWeights cw;
    cw.xy[0] = __fmul_rn(gx, gy);
    cw.xy[1] = __fmul_rn(fx, gy);
    cw.xy[2] = __fmul_rn(gx, fy);
    cw.xy[3] = __fmul_rn(fx, fy);
    cw.z[0] = gz;
    cw.z[1] = fz;
    return cw;
}

// seg of a neighbourhood whose eight labels agree: all eight weights accumulated from 0.
__device__ __forceinline__ float uniform_sum(const CornerWeights &cw) {
    float s = __fmul_rn(cw.xy[0], cw.z[0]);  // fma(xy, z, 0.0f)
#pragma unroll
    for (int c = 1; c < 8; c++) s = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], s);
    return s;
}

// seg[m] = the corner weights labelled m, accumulated in corner order from 0.
template <int M>
__device__ __forceinline__ void label_fractions(uint32_t word, const CornerWeights &cw, float seg[M]) {
#pragma unroll
    for (int m = 0; m < M; m++) seg[m] = 0.0f;
    if (uniform_word(word)) {
        const float s = uniform_sum(cw);
        const int L = (int)(word & 15u);
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m == L) seg[m] = s;
        return;
    }
    // two labels A (corner 0's) and B: one pass over the corners into two sums, each in corner order
    const uint32_t A = word & 15u;
    const uint32_t xa = word ^ (A * 0x11111111u);
    const uint32_t B = (word >> ((__ffs(xa) - 1) & ~3)) & 15u;
    const uint32_t xb = word ^ (B * 0x11111111u);
    const uint32_t za = ~(((xa & 0x77777777u) + 0x77777777u) | xa) & 0x88888888u;  // nibbles equal to A
    const uint32_t zb = ~(((xb & 0x77777777u) + 0x77777777u) | xb) & 0x88888888u;  // nibbles equal to B
    if ((za | zb) == 0x88888888u) {
        float sA = 0.0f, sB = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            if ((za >> (4 * c + 3)) & 1u)
                sA = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sA);
            else
                sB = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sB);
        }
#pragma unroll
        for (int m = 0; m < M; m++) seg[m] = (uint32_t)m == A ? sA : ((uint32_t)m == B ? sB : 0.0f);
    } else {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int L = (int)((word >> (4 * c)) & 15u);
#pragma unroll
            for (int m = 0; m < M; m++)
                if (m == L) seg[m] = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], seg[m]);
        }
    }
}

template <int M>
__device__ __forceinline__ void store_ad(float ad[M], int m_sel, float val) {
#pragma unroll
    for (int m = 0; m < M; m++)
        if (m == m_sel) ad[m] = val;
}
template <int M>
__device__ __forceinline__ float load_ad(const float ad[M], int m_sel) {
    float r = 0.0f;
#pragma unroll
    for (int m = 0; m < M; m++)
        if (m == m_sel) r = ad[m];
    return r;
}

// Shared memory of a block for the per-volume ray state of a multi-volume march: for each thread,
// kRayState values per volume in its own column [kRayState * NV][kBlockThreads].
constexpr int kRayState = 5;  // IJK direction x, y, z; entry and exit alpha
template <int NV>
constexpr int ray_state_floats() {
    return NV > 1 ? kRayState * NV * kBlockThreads : 1;
}

// The whole computation of one ray: pixel (u, v) of `view`, written to output view `vout`. `rs` is
// this thread's column of the block's ray-state array (unused for one volume).
template <int NV, int M>
__device__ __forceinline__ void render_ray(const SceneParams<NV> &p, const ViewRec<NV> &view, int u, int v,
                                           size_t vout, float *rs) {
    const float step = p.step;
    const int nmat = p.n_materials;

    // ---- ray setup (project_kernel.cu:218-234) ----
    const float uf = (float)u + 0.5f;
    const float vf = (float)v + 0.5f;
    float rx = ray_component(uf, view.w[0], vf, view.w[1], view.w[2]);
    float ry = ray_component(uf, view.w[3], vf, view.w[4], view.w[5]);
    float rz = ray_component(uf, view.w[6], vf, view.w[7], view.w[8]);
    const float ray_length = __fsqrt_rn(__fmaf_rn(rz, rz, __fmaf_rn(rx, rx, __fmul_rn(ry, ry))));
    const float inv_norm = __fdiv_rn(1.0f, ray_length);
    rx = __fmul_rn(rx, inv_norm);
    ry = __fmul_rn(ry, inv_norm);
    rz = __fmul_rn(rz, inv_norm);

    // ---- per-volume slab test (project_kernel.cu:265-323) ----
    float minA = ray_length, maxA = 0.0f;
    float rxi[NV], ryi[NV], rzi[NV], minv[NV], maxv[NV];
    bool trace[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) {
        trace[i] = false;
        minv[i] = 0.0f;
        maxv[i] = 0.0f;
        rxi[i] = ryi[i] = rzi[i] = 0.0f;
        if (!p.vol[i].enabled) continue;
        const float *A = view.vol[i].a;
        rxi[i] = dot3(A[0], rx, A[1], ry, A[2], rz);
        ryi[i] = dot3(A[3], rx, A[4], ry, A[5], rz);
        rzi[i] = dot3(A[6], rx, A[7], ry, A[8], rz);
        const float r3[3] = {rxi[i], ryi[i], rzi[i]};
        float mn = 0.0f;
        float mx = p.max_ray_length > 0.0f ? p.max_ray_length : __int_as_float(0x7f800000);
        bool ok = true;
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            if (!ok) break;
            const float s = view.vol[i].s[ax];
            const float hi = p.vol[i].hi[ax];
            if (0.0f != r3[ax]) {
                const float reci = __fdiv_rn(1.0f, r3[ax]);
                const float a0 = __fmul_rn(__fsub_rn(-0.5f, s), reci);
                const float a1 = __fmul_rn(__fsub_rn(hi, s), reci);
                mn = fmaxf(mn, fminf(a0, a1));
                mx = fminf(mx, fmaxf(a0, a1));
            } else if (-0.5f > s || s > hi) {
                ok = false;
            }
        }
        minv[i] = mn;
        maxv[i] = mx;
        if (!ok) continue;
        trace[i] = true;
        minA = fminf(minA, mn);
        maxA = fmaxf(maxA, mx);
    }
    // The per-volume state the march reads: in registers for one volume; for several, in shared
    // memory (this thread's column), which keeps the multi-volume march within its 64 registers.
    unsigned tmask = 0u;  // volumes traced
#pragma unroll
    for (int i = 0; i < NV; i++) {
        if (trace[i]) tmask |= 1u << i;
        if (NV > 1) {
            rs[(0 * NV + i) * kBlockThreads] = rxi[i];
            rs[(1 * NV + i) * kBlockThreads] = ryi[i];
            rs[(2 * NV + i) * kBlockThreads] = rzi[i];
            rs[(3 * NV + i) * kBlockThreads] = minv[i];
            rs[(4 * NV + i) * kBlockThreads] = maxv[i];
        }
    }
    auto RXI = [&](int i) -> float { return NV == 1 ? rxi[0] : rs[(0 * NV + i) * kBlockThreads]; };
    auto RYI = [&](int i) -> float { return NV == 1 ? ryi[0] : rs[(1 * NV + i) * kBlockThreads]; };
    auto RZI = [&](int i) -> float { return NV == 1 ? rzi[0] : rs[(2 * NV + i) * kBlockThreads]; };
    auto MINV = [&](int i) -> float { return NV == 1 ? minv[0] : rs[(3 * NV + i) * kBlockThreads]; };
    auto MAXV = [&](int i) -> float { return NV == 1 ? maxv[0] : rs[(4 * NV + i) * kBlockThreads]; };
    auto TRACE = [&](int i) -> bool { return ((tmask >> i) & 1u) != 0u; };

    const float span_steps = ceilf(__fdiv_rn(__fsub_rn(maxA, minA), step));
    const size_t plane = (size_t)p.width * (size_t)p.height;
    const size_t pix = (size_t)v * (size_t)p.width + (size_t)u;
    if (span_steps > (float)kMaxSteps || span_steps != span_steps) {
        // Only non-finite or absurd geometry gets here; report NaN rather than march for ever.
        const float nan = __int_as_float(0x7fc00000);
        p.intensity[vout * plane + pix] = nan;
        p.photon_prob[vout * plane + pix] = nan;
        if (p.area_density != nullptr)
            for (int m = 0; m < nmat; m++) p.area_density[(vout * nmat + m) * plane + pix] = nan;
        if (p.solid_angle != nullptr) p.solid_angle[vout * plane + pix] = nan;
        return;
    }
    const int num_steps = (int)span_steps;

    // live interval: union of the non-empty volume intervals
    float amin = __int_as_float(0x7f800000), amax = -__int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < NV; i++) {
        if (TRACE(i) && MINV(i) <= MAXV(i)) {
            amin = fminf(amin, MINV(i));
            amax = fmaxf(amax, MAXV(i));
        }
    }

    float ad[M];
#pragma unroll
    for (int m = 0; m < M; m++) ad[m] = 0.0f;
    const bool attenuate = p.attenuate != 0;
    const int air = p.air_index;
    if (attenuate) {
        const double pre = (double)__fdiv_rn(minA, step) * kAirDensity;
        store_ad<M>(ad, air, (float)((double)load_ad<M>(ad, air) + pre));
    }

    float alpha = minA;
    int t = 0;
    int t_end = num_steps;  // the march can stop here: no interval is open beyond it
    float alpha_stop = alpha;  // alpha at step t_end (set with t_end below)
    const bool carve = p.hit_alpha != nullptr;  // subtractive meshes: the reference's full march
    if (!p.full_march && !carve) {
        // Skip the steps before any interval opens and stop after the last one closes; the float32
        // alpha sequence is fast-forwarded exactly (drr_alpha.h), so later positions are unchanged.
        if (amin <= amax) {
            t = advance_alpha(&alpha, step, amin, num_steps, false);  // first alpha >= amin
            if (NV > 1 && t > 0) {  // replay one skipped step to seed the shared label cache
                alpha = minA;
                t = advance_alpha(&alpha, step, __int_as_float(0x7f800000), t - 1, false);
            }
            float a_end = alpha;
            t_end = t + advance_alpha(&a_end, step, amax, num_steps - t, true);  // first alpha > amax
            alpha_stop = a_end;
        } else {
            t = t_end = num_steps;  // no volume is ever sampled
        }
        if (attenuate) {
            float a = load_ad<M>(ad, air);
            for (int k = 0; k < t; k++) a = add_air(a);
            store_ad<M>(ad, air, a);
        }
    }

    // ---- the march (project_kernel.cu:398-553) ----
    float pb0 = __int_as_float(0x7fc00000), pb1 = pb0, pb2 = pb0;  // previous_coordinates (none yet)
    uint32_t word = 0;

    if (NV == 1 && !p.full_march && !carve) {
        // One volume between its entry and exit: n is 1 at every step and the label cache only
        // ever holds this volume's labels. The trapezoid half weights (project_kernel.cu:537) apply
        // to t = 0 and t = num_steps - 1 only, so those steps are peeled off the main loop.
        const VolConst &V = p.vol[0];
        // x and y travel as pairs (f32x2 arithmetic, the same roundings as the scalar operations)
        const float2 s2 = make_float2(view.vol[0].s[0], view.vol[0].s[1]);
        const float sz = view.vol[0].s[2];
        const float2 r2 = make_float2(RXI(0), RYI(0));
        const float rz0 = RZI(0);
        const float2 one2 = make_float2(1.0f, 1.0f), half2v = make_float2(0.5f, 0.5f);
        const float2 step2 = make_float2(step, step);
        float2 a2 = make_float2(alpha, alpha);  // alpha in both lanes
        int cur_m = -1;      // material whose accumulator is held in cur_ad
        float cur_ad = 0.0f;
        // Software pipelining of the label words: each step loads the word of the NEXT sample's
        // base, so the load's latency overlaps this sample's work and no lane branches to fetch.
        // With one volume the reference's cache always holds the current base's word, so loading
        // it for every sample is the same thing.
        float2 c2 = make_float2(0.0f, 0.0f), cb2 = make_float2(0.0f, 0.0f);
        float cz = 0.0f, cbz = 0.0f;
        uint32_t w_cur = 0;
        bool direct = false;  // every base of this march has a code-table entry without clamping
        if (t < t_end) {
            c2 = sub2_rn(fma2_rn(a2, r2, s2), one2);
            cz = __fsub_rn(__fmaf_rn(alpha, rz0, sz), 1.0f);
            cb2 = make_float2(floorf(c2.x), floorf(c2.y));
            cbz = floorf(cz);
            w_cur = fetch_label_code(V, cb2.x, cb2.y, cbz);
            // the last position whose code the march loads: one step past its last sample, at step
            // t_end, computed with the march's own operations
            const float2 e2 = sub2_rn(fma2_rn(make_float2(alpha_stop, alpha_stop), r2, s2), one2);
            const float ez = __fsub_rn(__fmaf_rn(alpha_stop, rz0, sz), 1.0f);
            direct = direct_bases(V, cb2, cbz, make_float2(floorf(e2.x), floorf(e2.y)), floorf(ez));
        }
        // `half` is std::true_type for the trapezoid half-weight samples, std::false_type otherwise:
        // a full-weight sample's weight 1 * rho is rho, so no multiply is issued for it. `dir` is
        // std::true_type where the march's bases need no clamping (`direct`): six fewer operations
        // per sample, the same codes.
        auto sample = [&](auto half, auto dir) {
            const float2 an2 = add2_rn(a2, step2);
            const float2 n2 = sub2_rn(fma2_rn(an2, r2, s2), one2);
            const float nz = __fsub_rn(__fmaf_rn(an2.x, rz0, sz), 1.0f);
            const float2 nb2 = make_float2(floorf(n2.x), floorf(n2.y));
            const float nbz = floorf(nz);
            const uint32_t w_next = decltype(dir)::value ? fetch_label_code_direct(V, nb2.x, nb2.y, nbz)
                                                         : fetch_label_code(V, nb2.x, nb2.y, nbz);
            const float2 f2 = sub2_rn(c2, cb2);
            const float fz = __fsub_rn(cz, cbz);
            const uint32_t code = w_cur;
            const int uni_label = (code & (kCodeGeneral | 0xFF00u)) == 0u ? (int)(code & 15u) : -1;
            const float2 g2 = sub2_rn(one2, f2);
            CornerWeights cw;
            cw.xy[0] = __fmul_rn(g2.x, g2.y);
            cw.xy[1] = __fmul_rn(f2.x, g2.y);
            cw.xy[2] = __fmul_rn(g2.x, f2.y);
            cw.xy[3] = __fmul_rn(f2.x, f2.y);
            cw.z[0] = __fsub_rn(1.0f, fz);
            cw.z[1] = fz;
            const float2 tc2 = add2_rn(c2, half2v);
            const float rho = tex3D<float>(V.density, tc2.x, tc2.y, __fadd_rn(cz, 0.5f));
            const float wr = decltype(half)::value ? __fmul_rn(0.5f, rho) : rho;
            if (uni_label >= 0) {
                const float s = uniform_sum(cw);
                if (uni_label != cur_m) {
                    if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                    cur_ad = load_ad<M>(ad, uni_label);
                    cur_m = uni_label;
                }
                cur_ad = __fmaf_rn(wr, s, cur_ad);
            } else {
                if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                cur_m = -1;
                // two labels A (corner 0's) and B: one pass over the corners into two sums, each
                // in corner order as the reference accumulates them; other materials get
                // fma(wr, 0, ad) = ad, exactly what the general path does for them
                if (!(code & kCodeGeneral)) {
                    const uint32_t A = code & 15u, B = (code >> 4) & 15u, mask = code >> 8;
                    float sA = 0.0f, sB = 0.0f;
#pragma unroll
                    for (int c = 0; c < 8; c++) {
                        if ((mask >> c) & 1u)
                            sB = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sB);
                        else
                            sA = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sA);
                    }
#pragma unroll
                    for (int m = 0; m < M; m++)
                        ad[m] = __fmaf_rn(wr, (uint32_t)m == A ? sA : ((uint32_t)m == B ? sB : 0.0f), ad[m]);
                } else {
                    word = general_label_word(V, code, cb2.x, cb2.y, cbz);  // three or more labels: the corners' own
                    float seg[M];
                    label_fractions<M>(word, cw, seg);
#pragma unroll
                    for (int m = 0; m < M; m++) ad[m] = __fmaf_rn(wr, seg[m], ad[m]);
                }
            }
            a2 = an2;
            alpha = an2.x;
            c2 = n2, cz = nz, cb2 = nb2, cbz = nbz;
            w_cur = w_next;
        };
        auto march = [&](auto dir) {
            if (t < t_end && t == 0) {
                sample(std::true_type{}, dir);
                ++t;
            }
            const bool last_half = t < t_end && t_end == num_steps;
            const int t_main = last_half ? t_end - 1 : t_end;
            // two samples per iteration: the loop-carried position and word then need no moves
#pragma unroll 2
            for (; t < t_main; ++t) sample(std::false_type{}, dir);
            if (last_half) {
                sample(std::true_type{}, dir);
                ++t;
            }
        };
        if (direct)
            march(std::true_type{});
        else
            march(std::false_type{});
        if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
    } else if (NV > 1 && !p.full_march && !carve) {
        // Several volumes between the first interval's entry and the last one's exit: the
        // reference's step (project_kernel.cu:394-553) with the same results, cheaper per step.
        //   * The set of volumes whose interval holds alpha changes only where alpha passes an
        //     interval end, so the priority resolution (project_kernel.cu:458-496), the 1/n weight
        //     and the mask of adding volumes are redone only there (`enter`: the next interval
        //     start ahead, `leave`: the nearest end of a live interval).
        //   * The label cache (project_kernel.cu:394-431) is keyed by the last base any enabled
        //     volume moved it to, so the key still follows every enabled volume each step. The word
        //     it holds is a function of (the volume that set the key, the key): when an adding volume
        //     set the key itself, that is its own word at its own base, which was loaded a step ahead;
        //     when another volume's base coincides with it (the reference's cross-volume quirk), the
        //     word is loaded from that volume's labels, as the reference's cache holds it. Two
        //     volumes' bases can only coincide where their IJK positions, affine in alpha, are within
        //     a voxel (plus a step, for the previous step's key) on every axis: an interval of alpha
        //     per pair, computed once per ray. Outside the hull of those intervals the key is always
        //     the adding volume's own base, so the other volumes are not followed there at all.
        //   * Uniform and two-label cells take the single-volume path's shortcuts (same additions).
        int cur = NV, n = 0;
        unsigned adds = 0;  // volumes adding at priority `cur` (no range re-check, project_kernel.cu:541)
        float wseg = 0.0f;  // 1 / n
        float enter = -__int_as_float(0x7f800000), leave = __int_as_float(0x7f800000);
        auto resolve = [&]() {
            cur = NV, n = 0;
            enter = __int_as_float(0x7f800000), leave = __int_as_float(0x7f800000);
#pragma unroll
            for (int i = 0; i < NV; i++) {
                if (!TRACE(i)) continue;
                if (alpha < MINV(i)) {
                    enter = fminf(enter, MINV(i));
                    continue;
                }
                if (alpha > MAXV(i)) continue;
                leave = fminf(leave, MAXV(i));
                const int pr = p.vol[i].priority;
                if (pr < cur) {
                    cur = pr;
                    n = 1;
                } else if (pr == cur) {
                    n += 1;
                }
            }
            adds = 0u;
            if (n != 0) {
#pragma unroll
                for (int i = 0; i < NV; i++)
                    if (TRACE(i) && p.vol[i].priority == cur) adds |= 1u << i;
            }
            wseg = n != 0 ? __fdiv_rn(1.0f, (float)n) : 0.0f;
        };
        // alpha range where two enabled volumes' bases may coincide (drr_coincide.h), rounded outwards
        float dlo, dhi;
        int last_vol = -1;  // the last enabled volume: it sets the key at the end of a step
        {
            bool en[NV];
            float sv[NV][3], rv[NV][3];
#pragma unroll
            for (int i = 0; i < NV; i++) {
                en[i] = p.vol[i].enabled != 0;
                if (en[i]) last_vol = i;
                sv[i][0] = view.vol[i].s[0], sv[i][1] = view.vol[i].s[1], sv[i][2] = view.vol[i].s[2];
                rv[i][0] = RXI(i), rv[i][1] = RYI(i), rv[i][2] = RZI(i);
            }
            double lo, hi;
            coincidence_range(NV, en, sv, rv, step, &lo, &hi);
            dlo = lo <= hi ? __double2float_rd(lo) : __int_as_float(0x7f800000);
            dhi = lo <= hi ? __double2float_ru(hi) : -__int_as_float(0x7f800000);
        }
        bool tracking = false;  // the previous step followed the key through every enabled volume
        float alpha_prev = __int_as_float(0x7fc00000);  // NaN before the first step: the key starts empty
        int key_vol = -1;  // volume whose labels the cached word comes from; the key is (pb0, pb1, pb2)
        uint32_t w_pre[NV];
        unsigned pre_ok = 0u;  // volumes whose code at this step's base was loaded a step ahead
#pragma unroll
        for (int i = 0; i < NV; i++) w_pre[i] = 0u;
        int cur_m = -1;  // material whose accumulator is held in cur_ad
        float cur_ad = 0.0f;
        auto msample = [&](float half) {
            if (alpha >= enter || alpha > leave) resolve();
            const float weight = __fmul_rn(wseg, half);  // fl(1/n) * 0.5 is exact
            if (n == 0 && attenuate) {
                if (cur_m == air)
                    cur_ad = add_air(cur_ad);
                else
                    store_ad<M>(ad, air, add_air(load_ad<M>(ad, air)));
            }
            const float an = __fadd_rn(alpha, step);
            const bool track = alpha >= dlo && alpha <= dhi;
            if (track && !tracking) {
                // entering the range: the key as the previous step left it, the last volume's base
#pragma unroll
                for (int i = 0; i < NV; i++) {
                    if (i != last_vol) continue;
                    const float *s = view.vol[i].s;
                    pb0 = floorf(__fsub_rn(__fmaf_rn(alpha_prev, RXI(i), s[0]), 1.0f));
                    pb1 = floorf(__fsub_rn(__fmaf_rn(alpha_prev, RYI(i), s[1]), 1.0f));
                    pb2 = floorf(__fsub_rn(__fmaf_rn(alpha_prev, RZI(i), s[2]), 1.0f));
                    key_vol = i;
                }
            }
            tracking = track;
            unsigned pre_next = 0u;
#pragma unroll
            for (int vol = 0; vol < NV; vol++) {
                if (!p.vol[vol].enabled) continue;
                if (!track && !((adds >> vol) & 1u)) continue;
                const float *s = view.vol[vol].s;
                const float px = __fsub_rn(__fmaf_rn(alpha, RXI(vol), s[0]), 1.0f);
                const float py = __fsub_rn(__fmaf_rn(alpha, RYI(vol), s[1]), 1.0f);
                const float pz = __fsub_rn(__fmaf_rn(alpha, RZI(vol), s[2]), 1.0f);
                const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
                if (track && (bx != pb0 || by != pb1 || bz != pb2)) {
                    pb0 = bx, pb1 = by, pb2 = bz;
                    key_vol = vol;
                }
                if (!((adds >> vol) & 1u)) continue;
                // the cached neighbourhood: this volume's own at its base, or the one of the volume
                // that set the key (the reference's cross-volume cache)
                uint32_t code;
                bool own = !track || key_vol == vol;
                if (own) {
                    code = (pre_ok >> vol) & 1u ? w_pre[vol] : fetch_label_code(p.vol[vol], bx, by, bz);
                } else {
                    code = 0u;
#pragma unroll
                    for (int i = 0; i < NV; i++)
                        if (i == key_vol) code = fetch_label_code(p.vol[i], pb0, pb1, pb2);
                }
                {  // this volume's code at the next step's base, loaded now
                    const float nx = __fsub_rn(__fmaf_rn(an, RXI(vol), s[0]), 1.0f);
                    const float ny = __fsub_rn(__fmaf_rn(an, RYI(vol), s[1]), 1.0f);
                    const float nz = __fsub_rn(__fmaf_rn(an, RZI(vol), s[2]), 1.0f);
                    w_pre[vol] = fetch_label_code(p.vol[vol], floorf(nx), floorf(ny), floorf(nz));
                    pre_next |= 1u << vol;
                }
                const CornerWeights cw = corner_weights(__fsub_rn(px, bx), __fsub_rn(py, by), __fsub_rn(pz, bz));
                const float rho = tex3D<float>(p.vol[vol].density, __fadd_rn(px, 0.5f), __fadd_rn(py, 0.5f),
                                               __fadd_rn(pz, 0.5f));
                const float wr = __fmul_rn(weight, rho);
                if ((code >> 8) == 0u) {
                    const int L = (int)(code & 15u);
                    const float su = uniform_sum(cw);
                    if (L != cur_m) {
                        if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                        cur_ad = load_ad<M>(ad, L);
                        cur_m = L;
                    }
                    cur_ad = __fmaf_rn(wr, su, cur_ad);
                } else {
                    if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                    cur_m = -1;
                    if (!(code & kCodeGeneral)) {
                        // two labels: the same additions as label_fractions makes for their word
                        const uint32_t A = code & 15u, B = (code >> 4) & 15u, mask = code >> 8;
                        float sA = 0.0f, sB = 0.0f;
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            if ((mask >> c) & 1u)
                                sB = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sB);
                            else
                                sA = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sA);
                        }
#pragma unroll
                        for (int m = 0; m < M; m++)
                            ad[m] = __fmaf_rn(wr, (uint32_t)m == A ? sA : ((uint32_t)m == B ? sB : 0.0f), ad[m]);
                    } else {
                        uint32_t w = 0u;
                        if (own) {
                            w = general_label_word(p.vol[vol], code, bx, by, bz);
                        } else {
#pragma unroll
                            for (int i = 0; i < NV; i++)
                                if (i == key_vol) w = general_label_word(p.vol[i], code, pb0, pb1, pb2);
                        }
                        float seg[M];
                        label_fractions<M>(w, cw, seg);
#pragma unroll
                        for (int m = 0; m < M; m++) ad[m] = __fmaf_rn(wr, seg[m], ad[m]);
                    }
                }
            }
            pre_ok = pre_next;
            alpha_prev = alpha;
            alpha = an;
        };
        if (t < t_end && t == 0) {
            msample(0.5f);
            ++t;
        }
        const bool last_half = t < t_end && t_end == num_steps;
        const int t_main = last_half ? t_end - 1 : t_end;
        // A stretch where one volume adds and no two bases can coincide is a single-volume march:
        // run it without the per-step interval and coincidence tests, its length counted in
        // advance with the exact float32 fast-forward (drr_alpha.h).
        auto single_stretch = [&]() -> bool {
            if (alpha >= enter || alpha > leave) resolve();
            if (n != 1 || __popc(adds) != 1 || (alpha >= dlo && alpha <= dhi)) return false;
            const float bound = alpha < dlo ? fminf(enter, dlo) : enter;
            float a = alpha;
            int kk = advance_alpha(&a, step, bound, t_main - t, false);  // samples below the next start
            a = alpha;
            kk = min(kk, advance_alpha(&a, step, leave, kk, true));       // and not past the end
            if (kk < 2) return false;
            // a is now the alpha one step past the stretch's last sample: the last position whose
            // label code the stretch loads
            const int v = __ffs(adds) - 1;
            const float vrx = RXI(v), vry = RYI(v), vrz = RZI(v);
            float vsx = view.vol[0].s[0], vsy = view.vol[0].s[1], vsz = view.vol[0].s[2];
#pragma unroll
            for (int i = 1; i < NV; i++)
                if (i == v) vsx = view.vol[i].s[0], vsy = view.vol[i].s[1], vsz = view.vol[i].s[2];
            const VolConst &Vv = p.vol[v];
            // n = 1 and full-weight samples: the weight fl(1 / 1) * rho is rho itself. x and y travel
            // as f32x2 pairs, as in the single-volume march.
            const float2 vr2 = make_float2(vrx, vry), vs2 = make_float2(vsx, vsy);
            const float2 one2 = make_float2(1.0f, 1.0f), half2v = make_float2(0.5f, 0.5f);
            const float2 step2 = make_float2(step, step);
            float2 a2 = make_float2(alpha, alpha);
            float2 c2 = sub2_rn(fma2_rn(a2, vr2, vs2), one2);
            float cz = __fsub_rn(__fmaf_rn(alpha, vrz, vsz), 1.0f);
            float2 cb2 = make_float2(floorf(c2.x), floorf(c2.y));
            float cbz = floorf(cz);
            // label codes, loaded a step ahead (the coincidence-free stretch needs no cache key);
            // without clamps where every base of the stretch has a table entry (direct_bases)
            uint32_t c_cur = fetch_label_code(Vv, cb2.x, cb2.y, cbz);
            const float2 e2 = sub2_rn(fma2_rn(make_float2(a, a), vr2, vs2), one2);
            const float ez = __fsub_rn(__fmaf_rn(a, vrz, vsz), 1.0f);
            const bool direct = direct_bases(Vv, cb2, cbz, make_float2(floorf(e2.x), floorf(e2.y)), floorf(ez));
            // two samples per iteration, as in the single-volume march (+11 % on the three-volume
            // batched workload, measured)
            auto stretch = [&](auto dir) {
#pragma unroll 2
            for (int k = 0; k < kk; k++) {
                const float2 an2 = add2_rn(a2, step2);
                const float2 n2 = sub2_rn(fma2_rn(an2, vr2, vs2), one2);
                const float nz = __fsub_rn(__fmaf_rn(an2.x, vrz, vsz), 1.0f);
                const float2 nb2 = make_float2(floorf(n2.x), floorf(n2.y));
                const float nbz = floorf(nz);
                const uint32_t c_next = decltype(dir)::value ? fetch_label_code_direct(Vv, nb2.x, nb2.y, nbz)
                                                             : fetch_label_code(Vv, nb2.x, nb2.y, nbz);
                const float2 f2 = sub2_rn(c2, cb2);
                const float fz = __fsub_rn(cz, cbz);
                const float2 g2 = sub2_rn(one2, f2);
                CornerWeights cw;
                cw.xy[0] = __fmul_rn(g2.x, g2.y);
                cw.xy[1] = __fmul_rn(f2.x, g2.y);
                cw.xy[2] = __fmul_rn(g2.x, f2.y);
                cw.xy[3] = __fmul_rn(f2.x, f2.y);
                cw.z[0] = __fsub_rn(1.0f, fz);
                cw.z[1] = fz;
                const float2 tc2 = add2_rn(c2, half2v);
                const float rho = tex3D<float>(Vv.density, tc2.x, tc2.y, __fadd_rn(cz, 0.5f));
                const float wr = rho;
                if ((c_cur & (kCodeGeneral | 0xFF00u)) == 0u) {
                    const int L = (int)(c_cur & 15u);
                    const float su = uniform_sum(cw);
                    if (L != cur_m) {
                        if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                        cur_ad = load_ad<M>(ad, L);
                        cur_m = L;
                    }
                    cur_ad = __fmaf_rn(wr, su, cur_ad);
                } else {
                    if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
                    cur_m = -1;
                    if (!(c_cur & kCodeGeneral)) {
                        const uint32_t A = c_cur & 15u, B = (c_cur >> 4) & 15u, mask = c_cur >> 8;
                        float sA = 0.0f, sB = 0.0f;
#pragma unroll
                        for (int c = 0; c < 8; c++) {
                            if ((mask >> c) & 1u)
                                sB = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sB);
                            else
                                sA = __fmaf_rn(cw.xy[c & 3], cw.z[c >> 2], sA);
                        }
#pragma unroll
                        for (int m = 0; m < M; m++)
                            ad[m] = __fmaf_rn(wr, (uint32_t)m == A ? sA : ((uint32_t)m == B ? sB : 0.0f), ad[m]);
                    } else {
                        float seg[M];
                        label_fractions<M>(general_label_word(Vv, c_cur, cb2.x, cb2.y, cbz), cw, seg);
#pragma unroll
                        for (int m = 0; m < M; m++) ad[m] = __fmaf_rn(wr, seg[m], ad[m]);
                    }
                }
                alpha_prev = alpha;
                alpha = an2.x;
                a2 = an2;
                c2 = n2, cz = nz, cb2 = nb2, cbz = nbz;
                c_cur = c_next;
            }
            };
            if (direct)
                stretch(std::true_type{});
            else
                stretch(std::false_type{});
            pre_ok = 0u;  // the words of the next step are loaded by msample
            tracking = false;
            t += kk;
            return true;
        };
        while (t < t_main) {
            if (single_stretch()) continue;
            msample(1.0f);
            ++t;
        }
        if (last_half) {
            msample(0.5f);
            ++t;
        }
        if (cur_m >= 0) store_ad<M>(ad, cur_m, cur_ad);
    } else {
        // DRR_FLAG_FULL_MARCH or subtractive meshes, any number of volumes: the reference's step. The
        // label cache is keyed by the last base any enabled volume moved it to
        // (project_kernel.cu:394-431), and a volume whose
        // base equals the key reads the cached word even if another volume's texture filled it. The
        // key therefore follows every enabled volume each step, but the word is only fetched when a
        // contributing volume needs it, from the texture of the volume that set the key: the same
        // words as the reference's eager fetches, without fetching for volumes that do not count.
        int key_vol = -1;     // volume whose texture the cached word comes from
        bool key_ok = false;  // the word of (key_vol, key) has been fetched
        int hidx[kMaxMeshLayers], hdepth[kMaxMeshLayers];
#pragma unroll
        for (int j = 0; j < kMaxMeshLayers; j++) hidx[j] = hdepth[j] = 0;
        for (; t < t_end; ++t) {
            // subtractive meshes (project_kernel.cu:498-519): count the crossings before alpha
            bool inside = false;
            if (carve) {
#pragma unroll
                for (int j = 0; j < kMaxMeshLayers; j++) {
                    if (j >= p.hit_layers) break;
                    const size_t base = ((size_t)j * plane + pix) * p.max_hits;
                    while (hidx[j] < p.max_hits) {
                        const int f = p.hit_facing[base + hidx[j]];
                        if (f == 0 || !(p.hit_alpha[base + hidx[j]] < alpha)) break;
                        hdepth[j] += f;
                        ++hidx[j];
                    }
                    inside |= hdepth[j] > 0;
                }
            }
            // priority resolution (project_kernel.cu:458-496) needs only alpha
            int cur = NV, n = 0;
#pragma unroll
            for (int i = 0; i < NV; i++) {
                if (!TRACE(i)) continue;
                if (alpha < MINV(i) || alpha > MAXV(i)) continue;
                const int pr = p.vol[i].priority;
                if (pr < cur) {
                    cur = pr;
                    n = 1;
                } else if (pr == cur) {
                    n += 1;
                }
            }
            float weight = 0.0f;
            if (n == 0) {
                if (attenuate && !inside) store_ad<M>(ad, air, add_air(load_ad<M>(ad, air)));
            } else {
                weight = __fdiv_rn(1.0f, (float)n);
                weight = __fmul_rn(weight, (0 == t || num_steps - 1 == t) ? 0.5f : 1.0f);
            }
#pragma unroll
            for (int vol = 0; vol < NV; vol++) {
                if (!p.vol[vol].enabled) continue;
                const float *s = view.vol[vol].s;
                const float px = __fsub_rn(__fmaf_rn(alpha, RXI(vol), s[0]), 1.0f);
                const float py = __fsub_rn(__fmaf_rn(alpha, RYI(vol), s[1]), 1.0f);
                const float pz = __fsub_rn(__fmaf_rn(alpha, RZI(vol), s[2]), 1.0f);
                const float bx = floorf(px), by = floorf(py), bz = floorf(pz);
                if (bx != pb0 || by != pb1 || bz != pb2) {
                    pb0 = bx;
                    pb1 = by;
                    pb2 = bz;
                    key_vol = vol;
                    key_ok = false;
                }
                // no range re-check, as in project_kernel.cu:541
                if (n != 0 && !inside && TRACE(vol) && p.vol[vol].priority == cur) {
                    if (!key_ok) {
#pragma unroll
                        for (int i = 0; i < NV; i++)
                            if (i == key_vol) word = fetch_label_word(p.vol[i], pb0, pb1, pb2);
                        key_ok = true;
                    }
                    float seg[M];
                    label_fractions<M>(word, corner_weights(__fsub_rn(px, bx), __fsub_rn(py, by), __fsub_rn(pz, bz)),
                                       seg);
                    const float rho = tex3D<float>(p.vol[vol].density, __fadd_rn(px, 0.5f), __fadd_rn(py, 0.5f),
                                                   __fadd_rn(pz, 0.5f));
                    const float wr = __fmul_rn(weight, rho);
#pragma unroll
                    for (int m = 0; m < M; m++) ad[m] = __fmaf_rn(wr, seg[m], ad[m]);
                }
            }
            alpha = __fadd_rn(alpha, step);
        }
    }
    if (attenuate) {
        float a = load_ad<M>(ad, air);
        for (; t < num_steps; ++t) a = add_air(a);
        const double post = (double)__fdiv_rn(__fsub_rn(ray_length, maxA), step) * kAirDensity;
        store_ad<M>(ad, air, (float)((double)a + post));
    }
#pragma unroll
    for (int m = 0; m < M; m++) ad[m] = __fmul_rn(ad[m], step);
    if (p.mesh_ad != nullptr) {
        // additive meshes (project_kernel.cu:569-579): after the step scaling, before the /10
        for (int k = 0; k < p.n_mesh; k++) {
            const float a = p.mesh_ad[(vout * p.n_mesh + k) * plane + pix];
            const int mm = p.mesh_mat[k];
#pragma unroll
            for (int m = 0; m < M; m++)
                if (m == mm) ad[m] = __fadd_rn(ad[m], a);
        }
    }
#pragma unroll
    for (int m = 0; m < M; m++) ad[m] = __fdiv_rn(ad[m], 10.0f);

    // ---- polychromatic attenuation (project_kernel.cu:637-646) ----
    float inten = 0.0f, prob = 0.0f;
    const float *__restrict__ mu = p.mu;
    for (int bin = 0; bin < p.n_bins; bin++) {
        float x = 0.0f;
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m < nmat) x = __fmaf_rn(ad[m], __ldg(mu + bin * nmat + m), x);
        const float pb = __fmul_rn(expf(-x), __ldg(p.pdf + bin));
        prob = __fadd_rn(prob, pb);
        inten = __fmaf_rn(__ldg(p.energies + bin), pb, inten);
    }

    p.intensity[vout * plane + pix] = inten;
    p.photon_prob[vout * plane + pix] = prob;
    if (p.area_density != nullptr) {
#pragma unroll
        for (int m = 0; m < M; m++)
            if (m < nmat) p.area_density[(vout * nmat + m) * plane + pix] = ad[m];
    }
    if (p.solid_angle != nullptr) p.solid_angle[vout * plane + pix] = pixel_solid_angle(view.w, u, v);
}

// Resident blocks per SM the forward kernels are compiled for: the march is issue- and latency-
// bound, and more warps hide its load and texture latency. Measured on GB300: 8 blocks of 128
// threads (64 registers) for one volume with 4 materials (+1 % over the compiler's 72 registers)
// and for three volumes with 4 materials (+25 % over its 96, with 72 bytes of spills). The other
// buckets take the most blocks that keep spills under ~80 bytes; 16 materials keep the
// compiler's choice.
template <int NV, int M>
constexpr int forward_min_blocks() {
    return M > 8 ? 1 : (NV <= 2 ? 8 : (NV == 3 ? (M <= 4 ? 8 : 7) : (M <= 4 ? 7 : 6)));
}

// Plain launch: one block per 16 x 8 pixel tile (each warp an 8 x 4 pixel sub-tile), z = view.
template <int NV, int M>
__global__ void __launch_bounds__(kBlockThreads, forward_min_blocks<NV, M>()) forward_kernel(const __grid_constant__ ForwardParams<NV> p) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int u = blockIdx.x * kTileW + ((warp & 1) << 3) + (lane & 7);
    const int v = blockIdx.y * kTileH + ((warp >> 1) << 2) + (lane >> 3);
    const int zv = blockIdx.z;
    if (u >= p.s.width || v >= p.s.height || zv >= p.n_views) return;
    __shared__ float rs[ray_state_floats<NV>()];
    render_ray<NV, M>(p.s, p.views[zv], u, v, (size_t)(p.view0 + zv), rs + threadIdx.x);
}

// Persistent launch: resident blocks take items_per_grab consecutive (view, tile) items at a time
// from an atomic counter, view-major so that neighbouring blocks share a view's part of the volume
// in L2. Rays of uneven length therefore balance across the GPU. Every block ends once the counter
// passes the last item; the loop has no waits.
template <int NV, int M>
__global__ void __launch_bounds__(kBlockThreads, forward_min_blocks<NV, M>()) forward_persistent_kernel(const __grid_constant__ PersistentParams<NV> p) {
    __shared__ unsigned int s_first;
    __shared__ float rs[ray_state_floats<NV>()];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int wx = p.warps_x;
    const int tile_w = 8 * wx, tile_h = 4 * (4 / wx);
    const unsigned int per_view = (unsigned int)p.tiles_x * (unsigned int)p.tiles_y;
    const unsigned int total = per_view * (unsigned int)p.n_views;
    const unsigned int grab = (unsigned int)p.items_per_grab;
    const int du = (warp % wx) * 8 + (lane & 7);
    const int dv = (warp / wx) * 4 + (lane >> 3);
    for (;;) {
        if (threadIdx.x == 0) s_first = atomicAdd(p.counter, grab);
        __syncthreads();
        const unsigned int first = s_first;
        __syncthreads();
        if (first >= total) break;
        const unsigned int last = first + grab < total ? first + grab : total;
        for (unsigned int it = first; it < last; ++it) {
            const unsigned int view = it / per_view, tile = it - view * per_view;
            const int u = (int)(tile % (unsigned int)p.tiles_x) * tile_w + du;
            const int v = (int)(tile / (unsigned int)p.tiles_x) * tile_h + dv;
            if (u < p.s.width && v < p.s.height) render_ray<NV, M>(p.s, p.views[view], u, v, (size_t)view, rs + threadIdx.x);
        }
    }
}

// Codes the labels of every 2x2x2 neighbourhood: the code of base b in [-2, n-1]^3 describes the labels
// at clamp(b + d, 0, n - 1), corner c = dx | dy << 1 | dz << 2 (the layout above kCodeGeneral).
__global__ void pack_labels_kernel(const uint8_t *__restrict__ labels, int ni, int nj, int nk, uint16_t *coded);
__global__ void count_general_kernel(const uint16_t *__restrict__ coded, int ni, int nj, int nk, uint32_t *counts);
__global__ void index_general_kernel(const uint8_t *__restrict__ labels, int ni, int nj, int nk, uint16_t *coded,
                                     const uint32_t *__restrict__ start, uint32_t *words);

// Host-side launcher, explicitly instantiated per (NV, M) in drr_inst_nv*.cu.
template <int NV, int M>
cudaError_t launch_forward(const ForwardParams<NV> &p, cudaStream_t stream);
template <int NV, int M>
cudaError_t launch_persistent(const PersistentParams<NV> &p, int grid_blocks, cudaStream_t stream);
template <int NV, int M>
int persistent_occupancy();

}  // namespace drr
