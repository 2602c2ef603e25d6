// rz_stroke.cuh -- the GPU stroker's unit table and arguments (rz_stroke.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

enum : uint32_t {
    STROKE_OFFSET = 0,     // seg: input segment; aux: 1 when reversed (the way back)
    STROKE_JOIN = 1,       // line_join before the OFFSET unit that follows
    STROKE_JOIN_CAP = 2,   // line_cap before the OFFSET unit that follows (an open subpath's turn)
    STROKE_CLOSE_FWD = 3,  // stroke_close of a closed subpath's forward list; seg / aux: its first / last segment
    STROKE_CLOSE_BWD = 4,  // stroke_close of the list back
    STROKE_CAPEND = 5,     // line_cap from the list's last piece to its first (open subpath)
};

enum : int { STROKE_JOIN_MITER = 0, STROKE_JOIN_BEVEL = 1, STROKE_JOIN_ROUND = 2 };
enum : int { STROKE_CAP_BUTT = 0, STROKE_CAP_SQUARE = 1, STROKE_CAP_ROUND = 2 };

struct StrokeUnit {
    uint32_t type;
    uint32_t seg;
    uint32_t aux;
    uint32_t list0;  // first unit of the unit's list (the pieces a join or close looks back over)
    uint32_t style;
};

// One input subpath of a stroke: its 4 m units start at unit `base`.
struct StrokeSub {
    uint64_t base;
    uint32_t s0, m;    // segments [s0, s0 + m)
    uint32_t closed;
    uint32_t style;
};

struct StrokeStyleDev {
    double width, miter;
    int32_t join, cap;
};

struct StrokeArgs {
    const StrokeUnit* units;
    uint32_t n_units;
    const StrokeStyleDev* styles;
    const uint8_t* kind;   // input segments (arc-free)
    const double* pts;
    uint32_t* counts;      // pieces per unit
    const uint64_t* off_start;  // OFFSET units: first piece in the compact buffer
    const uint64_t* fin_start;  // every unit: first piece in the output
    uint8_t* tmp_kind;     // compact buffer of OFFSET pieces
    double* tmp_pts;
    uint8_t* out_kind;     // the outline
    double* out_pts;
    int32_t strided;       // OFFSET pieces at kStrokeOffsetMax slots per unit (counts written by the emit pass)
    const uint32_t* order; // OFFSET units in launch order (cubics, then quads, then lines), or null: every unit
    uint32_t n_order;
    uint8_t* join_kind;    // the other (odd) units' pieces, 9 slots each, kept by the counting pass, or null
    double* join_pts;
};

constexpr int kStrokeOffsetMax = 36;  // 8 pieces of a cubic and 7 Round joins of up to 4 cubics

// A node of a curve's offset split tree (Segment::offset splits at 1/2 up to
// depth 3): curve t of the order list, depth d, index k, its control points.
struct StrokeNode {
    uint32_t t, k;
    int32_t d, kind;  // kind: 1 quad, 2 cubic
    double p[8];
};

// Scratch of the node-parallel offsets of the first n_curves entries of
// A.order (the quads and cubics): two node lists, the leaf list, their
// counters, and every leaf's offset piece at position k << (3 - d) of its curve.
struct StrokeNodes {
    StrokeNode* list[2];    // depth 1 (capacity 2 n_curves) and depth 2 (4 n_curves) nodes
    StrokeNode* leaves;     // capacity 8 n_curves
    uint32_t* counters;     // [0] list[0], [1] list[1], [2] leaves
    uint8_t* piece_kind;    // [n_curves * 8]
    double* piece_pts;      // [n_curves * 8 * 8]
    uint32_t* valid;        // [n_curves]: positions holding a piece
    uint32_t n_curves;
};

// The offsets of every OFFSET unit in A.order: the curves' split trees level by
// level (one thread per node), one thread per leaf for its offset, then one
// thread per unit assembles its pieces in order with the Round joins between
// them: counts (emit false) or counts and pieces at off_start (emit true).
// N's counters must be zero.
cudaError_t launch_stroke_nodes(const StrokeArgs& A, const StrokeNodes& N, cudaStream_t st);
cudaError_t launch_stroke_assemble(const StrokeArgs& A, const StrokeNodes& N, bool emit, cudaStream_t st);
// phase 2 / 3: the JOIN, CAP, CLOSE and CAPEND units' counts / pieces; 4: gather.
cudaError_t launch_stroke(const StrokeArgs& A, int phase, cudaStream_t st);
// The unit table of n_subs subpaths (n_units = the sum of their 4 m).
cudaError_t launch_stroke_units(const StrokeSub* subs, uint32_t n_subs, StrokeUnit* units, uint64_t n_units,
                                cudaStream_t st);

}  // namespace rz
