// Triangle setup of the meshlet rasterizer as device functions, shared by the raster kernels of
// libswr_gb300 and by the fragment stage of user shaders (include/swr/shader.cuh), which rebuilds a
// visible triangle's setup to hand its fragments the reference's barycentrics. Both run the same
// code, so both see the same bits.
//
// Each function restates the reference's per-lane arithmetic (src/SwRast/Rasterizer.cpp,
// Rasterizer.h, cited per function) with explicit round-to-nearest intrinsics.
#pragma once
#include <cstdint>

#include "approx14.h"
#include "device.cuh"

namespace swr {

struct Vtx { float x, y, z, w; };

// One lane of TrianglePacket (Rasterizer.h:145-161): snapped positions and depth / 1-over-w terms.
struct Setup {
    uint32_t Pos0, Pos1, Pos2;
    float Z0, Z1, Z2;
    float W0, W1, W2;  // 1 / w of the vertices (simd::perspective_div)
};

// TrianglePacket::GetBoundingBox / GetRenderBoundingBox (Rasterizer.cpp:331-351).
__device__ __forceinline__ void render_bbox(const Setup& t, int halfW, int halfH, uint32_t& bbMin, uint32_t& bbMax) {
    uint32_t minPos = __vmins2(__vmins2(t.Pos0, t.Pos1), t.Pos2);
    uint32_t maxPos = __vmaxs2(__vmaxs2(t.Pos0, t.Pos1), t.Pos2);
    minPos = srai16_4(minPos + 0x00070007u);  // 32-bit add, as the reference
    maxPos = srai16_4(maxPos + 0x00070007u);
    uint32_t vp = (uint32_t)halfW | ((uint32_t)halfH << 16);
    uint32_t x = __vmins2(__vmaxs2(__vadd2(minPos, vp), 0u), vp * 2);
    uint32_t y = __vmins2(__vmaxs2(__vadd2(maxPos, vp), 0u), vp * 2);
    bbMin = x & ~0x00030003u;
    bbMax = (y + 0x00030003u) & ~0x00030003u;
}

// ShadeMeshlet's vertex transform (Shading.cpp:295-298, simd::mul with w = 1, SIMD.h:457-464) by a
// column-major matrix m.
__device__ __forceinline__ float4 clip_transform(float x, float y, float z, const float* m) {
    float4 c;
    c.x = ffma(x, m[0], ffma(y, m[4], ffma(z, m[8], m[12])));
    c.y = ffma(x, m[1], ffma(y, m[5], ffma(z, m[9], m[13])));
    c.z = ffma(x, m[2], ffma(y, m[6], ffma(z, m[10], m[14])));
    c.w = ffma(x, m[3], ffma(y, m[7], ffma(z, m[11], m[15])));
    return c;
}

// A vertex after simd::perspective_div (SIMD.h:473-476): x/w, y/w, z/w and 1/w. The correctly
// rounded reciprocal is the same value as 1.0f / w.
struct Ndc { float x, y, z, rw; };
__device__ __forceinline__ Ndc project(float x, float y, float z, float w) {
    const float rw = __frcp_rn(w);
    return { fmul(x, rw), fmul(y, rw), fmul(z, rw), rw };
}

// The face test of TrianglePacket::Setup (Rasterizer.cpp:262-266): the float determinant of the
// projected vertices, negated for FrontCW or made absolute for None; the triangle is kept if > 0.
__device__ __forceinline__ bool front_facing(const Ndc& n0, const Ndc& n1, const Ndc& n2, int cullMode) {
    const float x0 = n0.x, y0 = n0.y, x1 = n1.x, y1 = n1.y, x2 = n2.x, y2 = n2.y;
    float det = fsub(fmul(fsub(x2, x0), fsub(y1, y0)), fmul(fsub(x0, x1), fsub(y0, y2)));
    if (cullMode != kCullFrontCCW) {
        bool flip = (cullMode == kCullFrontCW) ? true : (det < 0);
        det = flip ? -det : det;
    }
    return det > 0;
}

// TrianglePacket::Setup (Rasterizer.cpp:257-289) from projected vertices; returns the lane's keep bit.
__device__ __forceinline__ bool tri_setup_ndc(const Ndc& n0, const Ndc& n1, const Ndc& n2, int halfW, int halfH,
                                              int cullMode, Setup& t, uint32_t& bbMin, uint32_t& bbMax) {
    const float x0 = n0.x, y0 = n0.y, x1 = n1.x, y1 = n1.y, x2 = n2.x, y2 = n2.y;
    bool keep = front_facing(n0, n1, n2, cullMode);
    float fsx = (float)(halfW * 16), fsy = (float)(halfH * 16);
    int32_t ix0 = round2i(fmul(x0, fsx)), iy0 = round2i(fmul(y0, fsy));
    int32_t ix1 = round2i(fmul(x1, fsx)), iy1 = round2i(fmul(y1, fsy));
    int32_t ix2 = round2i(fmul(x2, fsx)), iy2 = round2i(fmul(y2, fsy));
    t.Pos0 = ((uint32_t)ix0 & 0xFFFF) | ((uint32_t)iy0 << 16);
    t.Pos1 = ((uint32_t)ix1 & 0xFFFF) | ((uint32_t)iy1 << 16);
    t.Pos2 = ((uint32_t)ix2 & 0xFFFF) | ((uint32_t)iy2 << 16);
    render_bbox(t, halfW, halfH, bbMin, bbMax);
    if (lo16(bbMin) >= lo16(bbMax) || hi16(bbMin) >= hi16(bbMax)) keep = false;
    t.Z0 = n0.z, t.Z1 = n1.z, t.Z2 = n2.z;
    t.W0 = n0.rw, t.W1 = n1.rw, t.W2 = n2.rw;
    return keep;
}

// tri_setup_ndc for a triangle already known to pass the face test (front_facing true): the same
// positions and bounding box; the keep bit is the box test alone.
__device__ __forceinline__ bool tri_setup_ndc_facing(const Ndc& n0, const Ndc& n1, const Ndc& n2, int halfW, int halfH,
                                                     Setup& t, uint32_t& bbMin, uint32_t& bbMax) {
    const float fsx = (float)(halfW * 16), fsy = (float)(halfH * 16);
    const int32_t ix0 = round2i(fmul(n0.x, fsx)), iy0 = round2i(fmul(n0.y, fsy));
    const int32_t ix1 = round2i(fmul(n1.x, fsx)), iy1 = round2i(fmul(n1.y, fsy));
    const int32_t ix2 = round2i(fmul(n2.x, fsx)), iy2 = round2i(fmul(n2.y, fsy));
    t.Pos0 = ((uint32_t)ix0 & 0xFFFF) | ((uint32_t)iy0 << 16);
    t.Pos1 = ((uint32_t)ix1 & 0xFFFF) | ((uint32_t)iy1 << 16);
    t.Pos2 = ((uint32_t)ix2 & 0xFFFF) | ((uint32_t)iy2 << 16);
    render_bbox(t, halfW, halfH, bbMin, bbMax);
    t.Z0 = n0.z, t.Z1 = n1.z, t.Z2 = n2.z;
    t.W0 = n0.rw, t.W1 = n1.rw, t.W2 = n2.rw;
    return lo16(bbMin) < lo16(bbMax) && hi16(bbMin) < hi16(bbMax);
}

// TrianglePacket::Setup from clip-space vertices (the clipper's output triangles).
__device__ __forceinline__ bool tri_setup(Vtx v0, Vtx v1, Vtx v2, int halfW, int halfH, int cullMode, Setup& t,
                                          uint32_t& bbMin, uint32_t& bbMax) {
    return tri_setup_ndc(project(v0.x, v0.y, v0.z, v0.w), project(v1.x, v1.y, v1.z, v1.w),
                         project(v2.x, v2.y, v2.z, v2.w), halfW, halfH, cullMode, t, bbMin, bbMax);
}

// ComputeEdge (Rasterizer.cpp:291-295), wrapping int32.
__device__ __forceinline__ int32_t compute_edge(int32_t a, int32_t x, int32_t b, int32_t y) {
    int32_t w = (int32_t)((uint32_t)a * (uint32_t)x + (uint32_t)b * (uint32_t)y);
    w = (int32_t)((uint32_t)w + ((a > 0 || (a == 0 && b > 0)) ? 0u : 0xFFFFFFFFu));
    return w >> 4;
}

// One lane of TriangleEdgeVars (Rasterizer.h:162-176): edge functions at pixel (0, 0), their steps,
// the depth plane, and rcpArea = 16 / det for the perspective terms.
struct Edges {
    int32_t E0, E1, E2;
    int32_t A12, B12, A20, B20, A01, B01;
    float Z0, Z10, Z20;
    float rcpArea;
    int32_t det;  // fixed-point determinant (> 0, or 0 for a triangle degenerate in fixed point)
};

// TriangleEdgeVars::Setup (Rasterizer.cpp:296-329).
__device__ __forceinline__ Edges edge_vars(const Setup& t, int halfW, int halfH) {
    Edges r;
    int32_t x0 = lo16(t.Pos0), y0 = hi16(t.Pos0);
    int32_t x1 = lo16(t.Pos1), y1 = hi16(t.Pos1);
    int32_t x2 = lo16(t.Pos2), y2 = hi16(t.Pos2);
    int32_t A01 = y1 - y0, B01 = x0 - x1;
    int32_t A12 = y2 - y1, B12 = x1 - x2;
    int32_t A20 = y0 - y2, B20 = x2 - x0;
    int32_t det = (int32_t)((uint32_t)B20 * (uint32_t)A01 - (uint32_t)B01 * (uint32_t)A20);
    if (det < 0) {
        A01 = -A01, B01 = -B01, A12 = -A12, B12 = -B12, A20 = -A20, B20 = -B20;
        det = -det;
    }
    int32_t sx = (int32_t)((uint32_t)(-halfW) << 4) + 8, sy = (int32_t)((uint32_t)(-halfH) << 4) + 8;
    r.E0 = compute_edge(A12, sx - x1, B12, sy - y1);
    r.E1 = compute_edge(A20, sx - x2, B20, sy - y2);
    r.E2 = compute_edge(A01, sx - x0, B01, sy - y0);
    r.A12 = A12, r.B12 = B12, r.A20 = A20, r.B20 = B20, r.A01 = A01, r.B01 = B01;
    // 16.0f / det: scaling the correctly rounded reciprocal by 16 is exact (|det| >= 1 or 0)
    r.rcpArea = fmul(16.0f, __frcp_rn(__int2float_rn(det)));
    r.Z0 = t.Z0;
    r.Z10 = fmul(fsub(t.Z1, t.Z0), r.rcpArea);
    r.Z20 = fmul(fsub(t.Z2, t.Z0), r.rcpArea);
    r.det = det;
    return r;
}

// The edge values of pixel (px, py) (Rasterizer.h:287-296): e0 | e1 | e2 >= 0 inside.
__device__ __forceinline__ void edge_values(const Edges& r, uint32_t px, uint32_t py, int32_t& e0, int32_t& e1, int32_t& e2) {
    e0 = (int32_t)((uint32_t)r.E0 + (uint32_t)r.A12 * px + (uint32_t)r.B12 * py);
    e1 = (int32_t)((uint32_t)r.E1 + (uint32_t)r.A20 * px + (uint32_t)r.B20 * py);
    e2 = (int32_t)((uint32_t)r.E2 + (uint32_t)r.A01 * px + (uint32_t)r.B01 * py);
}

// FragmentVars::Depth of DrawTriangle (Rasterizer.h:299) from the edge values (as floats).
__device__ __forceinline__ float fragment_depth(const Edges& r, float u, float v) {
    return ffma(u, r.Z10, ffma(v, r.Z20, r.Z0));
}

// Perspective-correct barycentrics of DrawTriangle (Rasterizer.h:300-317): from the edge values u, v
// (as floats), W0 and the W terms W0S/W1S/W2S = W * rcpArea; rcp14 is the exact table of
// VRCP14PS (approx14.h), refined by one Newton step. A clipped triangle's barycentrics are remapped
// to its source triangle by the TriangleClipData rows ru, rv (Rasterizer.cpp:455-458).
__device__ __forceinline__ void perspective_bary(float u, float v, float W0, float W0S, float W1S, float W2S, bool clipped,
                                                 const float* ru, const float* rv, float& bu, float& bv) {
    const float pw0 = ffma(fadd(u, v), -W0S, W0);
    const float w = ffma(u, W1S, ffma(v, W2S, pw0));
    float rcpW = swr_rcp14(w);                  // simd::approx_rcp (VRCP14PS, bit-exact)
    rcpW = fmul(rcpW, ffma(-w, rcpW, 2.0f));    // Newton-Raphson step
    bu = fmul(u, fmul(W1S, rcpW)), bv = fmul(v, fmul(W2S, rcpW));
    if (clipped) {
        const float cu = ffma(bu, ru[1], ffma(bv, ru[2], ru[0]));
        const float cv = ffma(bu, rv[1], ffma(bv, rv[2], rv[0]));
        bu = cu, bv = cv;
    }
}

// Per-vertex part of Clipper::ComputeClipCodes (Rasterizer.cpp:353-397): the six out-code bits and,
// in bit 6, the guard-band test |x| < w bx and |y| < w by. A triangle's codes combine its vertices'.
constexpr uint32_t kCodeInBand = 0x40u;
__device__ __forceinline__ uint32_t vertex_code(float4 q, float bx, float by) {
    uint32_t oc = 0;
    oc |= (q.x < -q.w) ? 1u : 0u;
    oc |= (q.x > q.w) ? 2u : 0u;
    oc |= (q.y < -q.w) ? 4u : 0u;
    oc |= (q.y > q.w) ? 8u : 0u;
    oc |= (q.z < -q.w) ? 16u : 0u;
    oc |= (q.z > q.w) ? 32u : 0u;
    if (fabsf(q.x) < fmul(q.w, bx) && fabsf(q.y) < fmul(q.w, by)) oc |= kCodeInBand;
    return oc;
}

// The polygon Clipper::ClipTriangles (Rasterizer.cpp:398-491) makes of one triangle against the
// planes in its out codes (x/y planes scaled by the guard band bx, by): vertices x, y, z, w and, with
// rows = 6, the barycentric coordinates u, v of the source triangle. The fan triangles are
// (idx[0], idx[i+1], idx[i+2]) for i + 2 < count.
struct ClipPoly {
    float V[6][16];
    uint8_t idx[16];
    uint32_t count;
};
// Returns false when a numerically non-convex polygon would exceed the buffers (which the reference
// only asserts, Rasterizer.cpp:441); the triangle is then dropped.
__device__ __forceinline__ bool clip_polygon(Vtx v0, Vtx v1, Vtx v2, uint32_t outcodes, float bx, float by, int rows,
                                             ClipPoly& P) {
    P.V[0][0] = v0.x, P.V[1][0] = v0.y, P.V[2][0] = v0.z, P.V[3][0] = v0.w;
    P.V[0][1] = v1.x, P.V[1][1] = v1.y, P.V[2][1] = v1.z, P.V[3][1] = v1.w;
    P.V[0][2] = v2.x, P.V[1][2] = v2.y, P.V[2][2] = v2.z, P.V[3][2] = v2.w;
    P.V[4][0] = 0.0f, P.V[4][1] = 1.0f, P.V[4][2] = 0.0f;
    P.V[5][0] = 0.0f, P.V[5][1] = 0.0f, P.V[5][2] = 1.0f;
    for (int k = 0; k < 16; k++) P.idx[k] = 0;
    P.idx[1] = 1, P.idx[2] = 2;
    uint32_t vertCount = 3, nextIdx = 3;
    const float guard[2] = { bx, by };
    for (uint32_t planeId = 0; planeId < 6; planeId++) {
        if (!((outcodes >> planeId) & 1)) continue;
        uint8_t out[16];
        uint32_t outCount = 0;
        float planeScale = planeId < 4 ? guard[planeId / 2] : 1.0f;
        for (uint32_t vi = 0; vi < vertCount; vi++) {
            uint32_t ia = P.idx[vi], ib = P.idx[(vi + 1) % vertCount];
            float aa = P.V[planeId / 2][ia], ab = P.V[planeId / 2][ib];
            if (planeId & 1) aa = -aa, ab = -ab;
            float da = fadd(aa, fmul(P.V[3][ia], planeScale));
            float db = fadd(ab, fmul(P.V[3][ib], planeScale));
            // A convex polygon gains at most one vertex per plane (at most 9 vertices, 12 new ones).
            if (outCount + 2 > 16 || nextIdx >= 16) return false;
            if (da >= 0) out[outCount++] = (uint8_t)ia;
            if ((da >= 0) != (db >= 0)) {
                float t = fdiv(da, fsub(da, db));
                for (int k = 0; k < rows; k++) P.V[k][nextIdx] = ffma(P.V[k][ib], t, ffma(-t, P.V[k][ia], P.V[k][ia]));
                out[outCount++] = (uint8_t)nextIdx++;
            }
        }
        if (vertCount < 3) break;  // stale count check, Rasterizer.cpp:443
        vertCount = outCount;
        for (int k = 0; k < 16; k++) P.idx[k] = out[k];
    }
    P.count = vertCount;
    return true;
}

// Fan triangle i of a clipped polygon as clip-space vertices, and its TriangleClipData rows
// (Rasterizer.cpp:455-458) when the polygon carries barycentrics.
__device__ __forceinline__ void clip_fan(const ClipPoly& P, uint32_t i, Vtx& a0, Vtx& a1, Vtx& a2, float* ru, float* rv) {
    const uint32_t i0 = P.idx[0], i1 = P.idx[i + 1], i2 = P.idx[i + 2];
    a0 = { P.V[0][i0], P.V[1][i0], P.V[2][i0], P.V[3][i0] };
    a1 = { P.V[0][i1], P.V[1][i1], P.V[2][i1], P.V[3][i1] };
    a2 = { P.V[0][i2], P.V[1][i2], P.V[2][i2], P.V[3][i2] };
    if (ru) {
        const float u0 = P.V[4][i0], w0 = P.V[5][i0];
        ru[0] = u0, ru[1] = fsub(P.V[4][i1], u0), ru[2] = fsub(P.V[4][i2], u0);
        rv[0] = w0, rv[1] = fsub(P.V[5][i1], w0), rv[2] = fsub(P.V[5][i2], w0);
    }
}

// Fields of a vis-buffer rank (make_rank): the global meshlet, the primitive, whether it is a
// clipper output and its fan index.
struct RankFields {
    uint32_t meshlet, prim, clipped, fan;
};
__device__ __forceinline__ RankFields decode_rank(uint32_t rank) {
    return { rank >> 11, ((rank >> 8) & 7) * 16u + ((rank >> 3) & 15), (rank >> 7) & 1, rank & 7 };
}

}  // namespace swr
