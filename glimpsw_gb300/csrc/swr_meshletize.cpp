// Meshlet building for imported meshes (the part of Scene::ImportGltf, Scene.cpp:196-276, that
// meshoptimizer's meshopt_buildMeshlets / meshopt_computeMeshletBounds do in the reference; that
// library is not available, so the grouping below is this project's own).
//
// Grouping: triangles are visited in the Morton order of their centroids. A meshlet grows from a
// seed by repeatedly taking, among the unassigned triangles that share a vertex with it, the one
// that shares the most vertices (ties: the earliest in Morton order), as long as it stays within
// 64 vertices and 128 triangles (ShadedMeshlet::MaxVertices / MaxPrims, Rasterizer.h:83). When no
// neighbour is left, the next unassigned triangle in Morton order continues the meshlet if it
// fits. A meshlet therefore closes only when nothing fits: it holds 128 triangles or at least 62
// vertices (hence at least 21 triangles), except possibly the last one.
//
// Bounds: a bounding sphere of the meshlet's vertices (Ritter's construction from the extreme
// points along the axes, radius widened by a relative 1e-6 so that every vertex lies inside after
// rounding) and a normal cone in meshoptimizer's convention (see below), which the backface-cone
// test of swr_cull_meshlets_ex reads; the reference's CullMeshlets reads only the sphere
// (Shading.cpp:797-809).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/swr_gb300.h"

swr_status swr_internal_fail(swr_status code, const char* msg);

namespace {

constexpr uint32_t kMaxVerts = 64, kMaxTris = 128;

// Meshlet record, Scene.h:15-30 (1728 bytes).
struct MeshletRecord {
    float BoundCenter[3];
    float BoundRadius;
    float ConeApex[3], ConeAxis[3];
    float ConeCutoff;
    uint8_t NumVertices, NumTriangles;
    uint8_t AlphaCutoff;
    uint32_t MaterialId;
    uint64_t TangentHandedness;
    alignas(64) float Positions[3][64];
    uint32_t TexCoords[64];
    uint32_t NormalTangents[64];
    uint8_t Indices[3][128];
};
static_assert(sizeof(MeshletRecord) == SWR_MESHLET_SIZE, "Meshlet record");

uint32_t spread_bits(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3FF;
    v = (v | (v << 16)) & 0x030000FF;
    v = (v | (v << 8)) & 0x0300F00F;
    v = (v | (v << 4)) & 0x030C30C3;
    v = (v | (v << 2)) & 0x09249249;
    return v;
}

struct Vec3 { double x, y, z; };

void bounding_sphere(const std::vector<Vec3>& p, Vec3& c, double& r) {
    // extreme points along each axis; the farthest pair seeds the sphere
    size_t lo[3] = { 0, 0, 0 }, hi[3] = { 0, 0, 0 };
    for (size_t i = 1; i < p.size(); i++) {
        const double v[3] = { p[i].x, p[i].y, p[i].z };
        for (int a = 0; a < 3; a++) {
            const double l[3] = { p[lo[a]].x, p[lo[a]].y, p[lo[a]].z }, h[3] = { p[hi[a]].x, p[hi[a]].y, p[hi[a]].z };
            if (v[a] < l[a]) lo[a] = i;
            if (v[a] > h[a]) hi[a] = i;
        }
    }
    auto d2 = [](const Vec3& a, const Vec3& b) {
        const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
        return dx * dx + dy * dy + dz * dz;
    };
    int best = 0;
    for (int a = 1; a < 3; a++)
        if (d2(p[lo[a]], p[hi[a]]) > d2(p[lo[best]], p[hi[best]])) best = a;
    const Vec3& a = p[lo[best]];
    const Vec3& b = p[hi[best]];
    c = { (a.x + b.x) * 0.5, (a.y + b.y) * 0.5, (a.z + b.z) * 0.5 };
    r = std::sqrt(d2(a, b)) * 0.5;
    for (const Vec3& q : p) {  // grow to contain every point
        const double d = std::sqrt(d2(q, c));
        if (d > r) {
            const double nr = (r + d) * 0.5, k = (nr - r) / d;
            c = { c.x + (q.x - c.x) * k, c.y + (q.y - c.y) * k, c.z + (q.z - c.z) * k };
            r = nr;
        }
    }
}

}  // namespace

extern "C" {

uint32_t swr_meshlet_bound(uint32_t num_triangles) { return num_triangles / 21 + 2; }

swr_status swr_build_meshlets(const swr_mesh_desc* mesh, void* out, uint32_t capacity, uint32_t* count) {
    if (!mesh || !count || (!out && capacity) || !mesh->positions || (!mesh->indices && mesh->num_triangles))
        return swr_internal_fail(SWR_EINVAL, "swr_build_meshlets: bad argument");
    const uint32_t nv = mesh->num_vertices, nt = mesh->num_triangles;
    for (uint64_t i = 0; i < (uint64_t)nt * 3; i++)
        if (mesh->indices[i] >= nv) return swr_internal_fail(SWR_EINVAL, "swr_build_meshlets: vertex index out of range");
    *count = 0;
    if (nt == 0) return SWR_OK;
    const float* P = mesh->positions;
    const uint32_t* I = mesh->indices;

    // Morton order of the triangle centroids over the mesh's bounding box
    float mn[3] = { P[0], P[1], P[2] }, mx[3] = { P[0], P[1], P[2] };
    for (uint32_t v = 0; v < nv; v++)
        for (int a = 0; a < 3; a++) mn[a] = std::min(mn[a], P[v * 3 + a]), mx[a] = std::max(mx[a], P[v * 3 + a]);
    std::vector<std::pair<uint32_t, uint32_t>> keyed(nt);
    for (uint32_t t = 0; t < nt; t++) {
        uint32_t code = 0;
        for (int a = 0; a < 3; a++) {
            const double c = ((double)P[I[t * 3] * 3 + a] + P[I[t * 3 + 1] * 3 + a] + P[I[t * 3 + 2] * 3 + a]) / 3.0;
            const double ext = (double)mx[a] - mn[a];
            const uint32_t q = ext > 0 ? (uint32_t)std::min(1023.0, std::max(0.0, (c - mn[a]) / ext * 1023.0)) : 0u;
            code |= spread_bits(q) << a;
        }
        keyed[t] = { code, t };
    }
    std::sort(keyed.begin(), keyed.end());
    std::vector<uint32_t> order(nt), rank(nt);
    for (uint32_t i = 0; i < nt; i++) order[i] = keyed[i].second, rank[keyed[i].second] = i;

    // vertex -> triangles (CSR)
    std::vector<uint32_t> start(nv + 1, 0), adj((size_t)nt * 3);
    for (uint64_t i = 0; i < (uint64_t)nt * 3; i++) start[I[i] + 1]++;
    for (uint32_t v = 0; v < nv; v++) start[v + 1] += start[v];
    {
        std::vector<uint32_t> fill(start.begin(), start.end() - 1);
        for (uint32_t t = 0; t < nt; t++)
            for (int k = 0; k < 3; k++) adj[fill[I[t * 3 + k]]++] = t;
    }

    std::vector<uint8_t> assigned(nt, 0);
    std::vector<uint32_t> vertMark(nv, UINT32_MAX), vertSlot(nv, 0), candMark(nt, UINT32_MAX);
    uint32_t cursor = 0, made = 0, left = nt;
    MeshletRecord* dst = (MeshletRecord*)out;
    std::vector<uint32_t> verts, tris, cands;
    while (left > 0) {
        if (made >= capacity) return swr_internal_fail(SWR_ECAPACITY, "swr_build_meshlets: output capacity too small");
        const uint32_t id = made;
        verts.clear(), tris.clear(), cands.clear();
        auto fits = [&](uint32_t t) {
            uint32_t add = 0;
            for (int k = 0; k < 3; k++) add += vertMark[I[t * 3 + k]] != id;
            return verts.size() + add <= kMaxVerts;
        };
        auto take = [&](uint32_t t) {
            assigned[t] = 1, left--;
            tris.push_back(t);
            for (int k = 0; k < 3; k++) {
                const uint32_t v = I[t * 3 + k];
                if (vertMark[v] != id) {
                    vertMark[v] = id, vertSlot[v] = (uint32_t)verts.size();
                    verts.push_back(v);
                    for (uint32_t j = start[v]; j < start[v + 1]; j++) {
                        const uint32_t n = adj[j];
                        if (!assigned[n] && candMark[n] != id) candMark[n] = id, cands.push_back(n);
                    }
                }
            }
        };
        while (tris.size() < kMaxTris) {
            // best neighbour: most shared vertices, then earliest in Morton order
            int bestShared = -1;
            uint32_t best = UINT32_MAX;
            size_t w = 0;
            for (size_t i = 0; i < cands.size(); i++) {
                const uint32_t t = cands[i];
                if (assigned[t]) continue;
                cands[w++] = t;
                int shared = 0;
                for (int k = 0; k < 3; k++) shared += vertMark[I[t * 3 + k]] == id;
                if (!fits(t)) continue;
                if (shared > bestShared || (shared == bestShared && rank[t] < rank[best])) bestShared = shared, best = t;
            }
            cands.resize(w);
            if (best == UINT32_MAX) {
                if (!cands.empty()) break;  // neighbours remain but none fits
                while (cursor < nt && assigned[order[cursor]]) cursor++;
                if (cursor == nt || !fits(order[cursor])) break;
                best = order[cursor];
            }
            take(best);
        }

        MeshletRecord& m = dst[made++];
        memset(&m, 0, sizeof(m));
        m.NumVertices = (uint8_t)verts.size();
        m.NumTriangles = (uint8_t)tris.size();
        m.MaterialId = mesh->material_id;
        m.AlphaCutoff = mesh->alpha_cutoff;
        std::vector<Vec3> pts(verts.size());
        for (size_t i = 0; i < verts.size(); i++) {
            const uint32_t v = verts[i];
            for (int a = 0; a < 3; a++) m.Positions[a][i] = P[v * 3 + a];
            pts[i] = { P[v * 3], P[v * 3 + 1], P[v * 3 + 2] };
            if (mesh->texcoords) m.TexCoords[i] = mesh->texcoords[v];
            if (mesh->normal_tangents) m.NormalTangents[i] = mesh->normal_tangents[v];
            if (mesh->tangent_signs && mesh->tangent_signs[v]) m.TangentHandedness |= 1ull << i;
        }
        Vec3 axis = { 0, 0, 0 };
        std::vector<Vec3> normals(tris.size());
        for (size_t i = 0; i < tris.size(); i++) {
            const uint32_t t = tris[i];
            for (int k = 0; k < 3; k++) m.Indices[k][i] = (uint8_t)vertSlot[I[t * 3 + k]];
            const Vec3 &a = pts[vertSlot[I[t * 3]]], &b = pts[vertSlot[I[t * 3 + 1]]], &c = pts[vertSlot[I[t * 3 + 2]]];
            const Vec3 e1 = { b.x - a.x, b.y - a.y, b.z - a.z }, e2 = { c.x - a.x, c.y - a.y, c.z - a.z };
            Vec3 n = { e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x };
            const double len = std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
            if (len > 0) n = { n.x / len, n.y / len, n.z / len };
            normals[i] = n;
            axis = { axis.x + n.x, axis.y + n.y, axis.z + n.z };
        }
        Vec3 c;
        double r;
        bounding_sphere(pts, c, r);
        r = r * (1.0 + 1e-6) + 1e-30;
        m.BoundCenter[0] = (float)c.x, m.BoundCenter[1] = (float)c.y, m.BoundCenter[2] = (float)c.z;
        float rf = (float)r;
        for (const Vec3& q : pts) {  // the float centre and radius must still contain every vertex
            const double dx = q.x - m.BoundCenter[0], dy = q.y - m.BoundCenter[1], dz = q.z - m.BoundCenter[2];
            const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
            while ((double)rf < d) rf = std::nextafter(rf, INFINITY);
        }
        m.BoundRadius = rf;
        // Normal cone in meshoptimizer's convention (every triangle faces away from a camera at e when
        // dot(normalize(apex - e), axis) >= cutoff): axis = normalised mean normal; with m the least
        // cosine between a normal and the axis, cutoff = sqrt(1 - m^2), and the apex is the point
        // centre - t*axis behind every triangle's plane. m <= 0.1 gives the degenerate cone
        // (cutoff 1, axis 0, apex = centre), which never culls.
        const double al = std::sqrt(axis.x * axis.x + axis.y * axis.y + axis.z * axis.z);
        if (al > 0) axis = { axis.x / al, axis.y / al, axis.z / al };
        double mindp = al > 0 ? 1.0 : -1.0;
        for (const Vec3& n : normals) mindp = std::min(mindp, n.x * axis.x + n.y * axis.y + n.z * axis.z);
        m.ConeApex[0] = m.BoundCenter[0], m.ConeApex[1] = m.BoundCenter[1], m.ConeApex[2] = m.BoundCenter[2];
        m.ConeCutoff = 1.0f;
        if (mindp > 0.1) {
            const Vec3 cc = { m.BoundCenter[0], m.BoundCenter[1], m.BoundCenter[2] };
            double t = 0.0;
            for (size_t i = 0; i < tris.size(); i++) {
                const Vec3& n = normals[i];
                const Vec3& a = pts[vertSlot[I[tris[i] * 3]]];
                const double dn = n.x * axis.x + n.y * axis.y + n.z * axis.z;
                const double dc = (cc.x - a.x) * n.x + (cc.y - a.y) * n.y + (cc.z - a.z) * n.z;
                if (dn > 0) t = std::max(t, dc / dn);
            }
            m.ConeApex[0] = (float)(cc.x - axis.x * t), m.ConeApex[1] = (float)(cc.y - axis.y * t);
            m.ConeApex[2] = (float)(cc.z - axis.z * t);
            m.ConeAxis[0] = (float)axis.x, m.ConeAxis[1] = (float)axis.y, m.ConeAxis[2] = (float)axis.z;
            m.ConeCutoff = (float)std::sqrt(std::max(0.0, 1.0 - mindp * mindp));
        }
    }
    *count = made;
    return SWR_OK;
}

}  // extern "C"
