// Host-side 4x4 matrix helpers used wherever the pipeline derives matrices from the caller's
// (the frustum planes of ShadingContext::CullMeshlets, Shading.cpp:779-794, and
// GetInverseScreenProjMatrix, Camera.h:140-146). The reference uses glm for these; this
// header restates the same definitions in plain float32 code with a fixed operation order,
// so every consumer of a given camera derives bit-identical matrices. Column-major storage,
// m[c * 4 + r] = column c, row r, as glm lays out mat4.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

namespace swr_hostmath {

// a * b, each output summed over k in ascending order.
inline void mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; c++) {
        for (int row = 0; row < 4; row++) {
            float s = a[0 * 4 + row] * b[c * 4 + 0];
            s = s + a[1 * 4 + row] * b[c * 4 + 1];
            s = s + a[2 * 4 + row] * b[c * 4 + 2];
            s = s + a[3 * 4 + row] * b[c * 4 + 3];
            r[c * 4 + row] = s;
        }
    }
    memcpy(out, r, sizeof(r));
}

// Inverse by Gauss-Jordan elimination with partial pivoting in double precision, rounded to
// float at the end. Returns false for a singular matrix (out is then left unchanged).
inline bool mat4_inverse(const float* m, float* out) {
    double a[4][8];
    for (int r = 0; r < 4; r++) {
        for (int c = 0; c < 4; c++) a[r][c] = (double)m[c * 4 + r];
        for (int c = 0; c < 4; c++) a[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
        if (a[piv][col] == 0.0) return false;
        if (piv != col)
            for (int c = 0; c < 8; c++) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
        double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f = a[r][col];
            if (f == 0.0) continue;
            for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[c * 4 + r] = (float)a[r][4 + c];
    return true;
}

// m * translation(v): column 3 becomes m0*v.x + m1*v.y + m2*v.z + m3.
inline void mat4_translate(float* m, float vx, float vy, float vz) {
    for (int r = 0; r < 4; r++) {
        float s = m[0 * 4 + r] * vx;
        s = s + m[1 * 4 + r] * vy;
        s = s + m[2 * 4 + r] * vz;
        s = s + m[3 * 4 + r];
        m[3 * 4 + r] = s;
    }
}
// m * scale(v): columns 0..2 scaled.
inline void mat4_scale(float* m, float sx, float sy, float sz) {
    for (int r = 0; r < 4; r++) {
        m[0 * 4 + r] = m[0 * 4 + r] * sx;
        m[1 * 4 + r] = m[1 * 4 + r] * sy;
        m[2 * 4 + r] = m[2 * 4 + r] * sz;
    }
}

// GetInverseScreenProjMatrix (Camera.h:140-146) with the default half-pixel offset: maps
// (pixel x, pixel y, ndc z, 1) to world space.
inline bool inverse_screen_proj(const float* worldToClip, uint32_t width, uint32_t height, float* out) {
    float inv[16];
    if (!mat4_inverse(worldToClip, inv)) return false;
    mat4_translate(inv, -1.0f, -1.0f, 0.0f);
    mat4_scale(inv, 2.0f / (float)width, 2.0f / (float)height, 1.0f);
    mat4_translate(inv, 0.5f, 0.5f, 0.0f);
    memcpy(out, inv, sizeof(inv));
    return true;
}

// Gribb & Hartmann frustum planes of CullMeshlets (Shading.cpp:779-791): for i = 0..2,
// plane 2i = row3 + row_i, plane 2i+1 = row3 - row_i, each divided by |xyz|.
inline void frustum_planes(const float* objectToClip, float planes[6][4]) {
    for (int i = 0; i < 3; i++) {
        float a[4], b[4];
        for (int k = 0; k < 4; k++) {
            float r3 = objectToClip[k * 4 + 3], ri = objectToClip[k * 4 + i];
            a[k] = r3 + ri;
            b[k] = r3 - ri;
        }
        float la = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        float lb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        for (int k = 0; k < 4; k++) {
            planes[i * 2 + 0][k] = a[k] / la;
            planes[i * 2 + 1][k] = b[k] / lb;
        }
    }
}

// Camera centre in object space for backface-cone culling: the point that objectToClip maps to
// clip x = y = w = 0, i.e. the null vector of its x, y and w rows (solved in double). Returns false
// when the cone test does not apply: an affine (orthographic) or singular projection, or one that
// mirrors the screen so that FrontCCW keeps triangles whose (b-a)x(c-a) normal points away from
// the camera. The orientation is read off a small triangle placed in front of the camera with its
// normal towards it, projected and tested with TrianglePacket::Setup's determinant
// (Rasterizer.cpp:262-266): it must come out front-facing (det > 0).
inline bool cone_camera(const float* m, float eye[3]) {
    const int rows[3] = { 0, 1, 3 };
    double A[3][3], b[3];
    for (int i = 0; i < 3; i++) {
        for (int c = 0; c < 3; c++) A[i][c] = (double)m[c * 4 + rows[i]];
        b[i] = -(double)m[3 * 4 + rows[i]];
    }
    auto det3 = [](double M[3][3]) {
        return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    };
    double scale = 0;
    for (int i = 0; i < 3; i++)
        for (int c = 0; c < 3; c++) scale = fmax(scale, fabs(A[i][c]));
    const double d = det3(A);
    if (!(fabs(d) > 1e-12 * scale * scale * scale)) return false;
    double e[3];
    for (int c = 0; c < 3; c++) {  // Cramer's rule
        double M[3][3];
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) M[i][k] = (k == c) ? b[i] : A[i][k];
        e[c] = det3(M) / d;
    }
    // w grows along g (the w row); a triangle at e + g/|g| with normal -g faces the camera.
    double g[3] = { A[2][0], A[2][1], A[2][2] };
    const double gl = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    if (!(gl > 0)) return false;
    for (int k = 0; k < 3; k++) g[k] /= gl;
    const double h[3] = { fabs(g[0]) < 0.9 ? 1.0 : 0.0, fabs(g[0]) < 0.9 ? 0.0 : 1.0, 0.0 };
    double u[3] = { h[1] * g[2] - h[2] * g[1], h[2] * g[0] - h[0] * g[2], h[0] * g[1] - h[1] * g[0] };
    const double ul = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int k = 0; k < 3; k++) u[k] /= ul;
    const double v[3] = { g[1] * u[2] - g[2] * u[1], g[2] * u[0] - g[0] * u[2], g[0] * u[1] - g[1] * u[0] };  // g x u
    // vertices q, q + v/100, q + u/100: (v x u) = -g, so the normal points at the camera
    const double dist = 1.0 + sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * 1e-3;
    double P[3][3];
    for (int k = 0; k < 3; k++) {
        const double q = e[k] + g[k] * dist;
        P[0][k] = q, P[1][k] = q + v[k] * dist * 0.01, P[2][k] = q + u[k] * dist * 0.01;
    }
    double nx[3], ny[3];
    for (int i = 0; i < 3; i++) {
        double c4[4];
        for (int r = 0; r < 4; r++)
            c4[r] = (double)m[0 * 4 + r] * P[i][0] + (double)m[1 * 4 + r] * P[i][1] + (double)m[2 * 4 + r] * P[i][2] +
                    (double)m[3 * 4 + r];
        if (!(c4[3] > 0)) return false;
        nx[i] = c4[0] / c4[3], ny[i] = c4[1] / c4[3];
    }
    const double det = (nx[2] - nx[0]) * (ny[1] - ny[0]) - (nx[0] - nx[1]) * (ny[0] - ny[2]);
    if (!(det > 0)) return false;
    for (int k = 0; k < 3; k++) eye[k] = (float)e[k];
    return true;
}

// glm::length(vec3(m[0])): uniform-scale estimate of a model matrix (Shading.cpp:793).
inline float column0_length(const float* m) { return sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]); }

}  // namespace swr_hostmath
