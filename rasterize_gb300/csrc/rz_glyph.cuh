// rz_glyph.cuh -- data layout of the glyph pipeline (rz_glyph.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rz_device.cuh"
#include "rz_kernels.cuh"

namespace rz {

// Shared-memory band of one k_glyph_cover CTA (4 CTAs per SM).
#ifndef RZ_GLYPH_BAND_KB
#define RZ_GLYPH_BAND_KB 48
#endif
constexpr int kGlyphBandBytes = RZ_GLYPH_BAND_KB * 1024;
constexpr int kGlyphBandFloats = kGlyphBandBytes / 4;

// Per-slot record kept between the passes.
struct __align__(16) GlyphRec {
    SegRec rec;    // 60 bytes: fixed-point segment (rz_device.cuh)
    uint32_t tag;  // state << 30 | owning path, as the band kernel's SlotRec
};
static_assert(sizeof(GlyphRec) == 64, "glyph record layout");

// Per-slot decision coefficients (FlatCoef and its quantisation bound).
struct __align__(8) GlyphCoef {
    float a2x, a2y, a3x, a3y, mag, qerr;
};

struct GlyphDev {
    BatchDev b;                // the batch: inputs, masks, output, error word, thresholds
    GlyphRec* recs;            // [n_slots]
    GlyphCoef* coefs;          // [n_slots]
    uint32_t* chain;           // [n_slots + 1] chain vertices per slot, then their exclusive prefix
    unsigned long long* code;  // [n_slots] pre-order tree code of each slot
    uint32_t* path_flags;      // [n_paths] bit 0: the path has slots the fixed-point route cannot take
    int4* vtx;                 // [vtx_cap] chain vertices
    uint32_t vtx_cap;
    void* paths;               // [n_paths] per-path descriptors of the cover items (glyph_path_bytes() each)
    int32_t walk_slots;        // slots each lane of the tree walk takes (1..16; 32 of them per warp)
};

constexpr int kWalkSlotsDefault = 4;

cudaError_t init_glyph_kernels();
int glyph_cover_occupancy();
uint64_t glyph_path_bytes();
cudaError_t launch_glyph_walk(const GlyphDev& g, cudaStream_t st);
cudaError_t launch_glyph_emit(const GlyphDev& g, cudaStream_t st);
cudaError_t launch_glyph_cover(const GlyphDev& g, const WorkItem* items, int n_items, int32_t* queue, int grid,
                               cudaStream_t st);

}  // namespace rz
