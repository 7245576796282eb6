// integrand.h — seeded analytic integrands that stand in for the reference's
// OptiX ray-generation programs (SDK/cuda/whitted.cu:164-293, SDK/cuda/direct.cu:116-152).
//
// An integrand maps one MDAS sample coordinate (AoS, `dim` floats: image x in
// [0, scaleX), image y in [0, scaleY), then the non-image dimensions in [0, 1))
// to an RGB radiance, exactly like `__raygen__pinhole_mdas_*` fills
// `params.sample_values[sample_offset + i]`.
//
// The code uses only correctly rounded IEEE-754 binary32 operations with
// explicit fused multiply-adds (see ieee_math.h), so the device build (compiled
// without contraction, -fmad=false) and a host build (-ffp-contract=off) give
// the same bits.  That lets every MDAS parity check assume identical sample
// values.
#pragma once

#include "ieee_math.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef MDAS_SCENE_DISCS_MB
#define MDAS_SCENE_DISCS_MB 0      // (x, y, t): 2-D discs moving linearly over the shutter
#define MDAS_SCENE_DISCS_DOF 1     // (x, y, u, v): fronto-parallel discs behind a thin lens
#define MDAS_SCENE_DISCS_MBDOF 2   // (x, y, t, u, v): both
#define MDAS_SCENE_DIRECT_LIGHT 3  // (x, y, u, v): ground + spheres lit by a rectangular light
#endif

// Floats per primitive.  Discs: [cx, cy, z, r, vx, vy, z/focal, r*r, R, G, B, 0];
// depth-of-field scenes list their discs by increasing depth (stable order).
// Spheres: [cx, cy, cz, r, 0, 0, 1/r, r*r, 0, 0, 0, 0].
#define MDAS_PRIM_STRIDE 12

typedef struct MdasScene {
    int kind;
    int dim;
    int count;
    int reserved;
    float scaleX, scaleY;        // sample-space extent of the image axes
    float background;            // grey for rays that hit nothing
    float filmHalfW, filmHalfH;  // tan(fovy/2) * aspect, tan(fovy/2)
    float focalDistance;
    float lensRadius;
    float eye[3];
    float U[3], V[3], W[3];      // pinhole basis for the lit scene: d = nx*U + ny*V + W
    float lightCorner[3];        // rectangle corner; edges along +x and +y
    float lightSize;
    float emission;
    float albedo;
} MdasScene;

#ifdef __cplusplus
}
#endif

MDAS_HD float mdas_dot3(const float* a, const float* b) {
    return mdas_fma(a[0], b[0], mdas_fma(a[1], b[1], a[2] * b[2]));
}

// Concentric square-to-disc mapping of (u, v) in [0,1)^2, as the reference's
// depth-of-field ray generation does it (SDK/cuda/whitted.cu:186-206):
// r = the larger offset, theta = pi/4 * (b/a) or pi/2 - pi/4 * (a/b).
MDAS_HD void mdas_concentric(float u, float v, float radius, float* lx, float* ly) {
    const float ax = (u + u) - 1.0f;
    const float ay = (v + v) - 1.0f;
    if (ax == 0.0f && ay == 0.0f) {
        *lx = 0.0f;
        *ly = 0.0f;
        return;
    }
    float s, c;
    if (fabsf(ax) > fabsf(ay)) {
        const float rr = radius * ax;
        mdas_sincos_quarter(0.785398163f * (ay / ax), &s, &c);
        *lx = rr * c;
        *ly = rr * s;
    } else {
        // theta = pi/2 - phi: cos(theta) = sin(phi), sin(theta) = cos(phi)
        const float rr = radius * ay;
        mdas_sincos_quarter(0.785398163f * (ax / ay), &s, &c);
        *lx = rr * s;
        *ly = rr * c;
    }
}

// Motion-blur disc p covers image point (px, py) at shutter time t.
MDAS_HD int mdas_disc_mb_covers(const float* p, float px, float py, float t) {
    const float dx = px - mdas_fma(p[4], t, p[0]);
    const float dy = py - mdas_fma(p[5], t, p[1]);
    return mdas_fma(dx, dx, dy * dy) <= p[7];
}

MDAS_HD void mdas_shade_discs_mb(const MdasScene* sc, const float* prims, const float* c, float* out) {
    const float px = c[0] / sc->scaleX;
    const float py = c[1] / sc->scaleY;
    const float t = c[2];
    float R = sc->background, G = sc->background, B = sc->background;
    // the last listed covering disc wins: scan from the back, stop at the first cover
    for (int k = sc->count - 1; k >= 0; --k) {
        const float* p = prims + MDAS_PRIM_STRIDE * k;
        if (mdas_disc_mb_covers(p, px, py, t)) {
            R = p[8];
            G = p[9];
            B = p[10];
            break;
        }
    }
    out[0] = R;
    out[1] = G;
    out[2] = B;
}

// Thin-lens ray of sample c (layout of mdas_shade_discs_dof): shutter time t,
// lens point (lx, ly) and the offset (wx, wy) from the lens point to the
// pinhole ray's point on the focal plane.
MDAS_HD void mdas_dof_ray(const MdasScene* sc, const float* c, int moving, float* t, float* lx, float* ly, float* wx,
                          float* wy) {
    const float px = c[0] / sc->scaleX;
    const float py = c[1] / sc->scaleY;
    *t = moving ? c[2] : 0.0f;
    const float u = moving ? c[3] : c[2];
    const float v = moving ? c[4] : c[3];
    const float nx = (px + px) - 1.0f;
    const float ny = (py + py) - 1.0f;
    mdas_concentric(u, v, sc->lensRadius, lx, ly);
    *wx = sc->focalDistance * (nx * sc->filmHalfW) - *lx;
    *wy = sc->focalDistance * (ny * sc->filmHalfH) - *ly;
}

// Fronto-parallel disc p covers the lens ray at its depth: the ray meets the
// disc's plane at lens point + (depth / focal) * offset.
MDAS_HD int mdas_disc_dof_covers(const float* p, float lx, float ly, float wx, float wy, float t, int moving) {
    const float hx = mdas_fma(p[6], wx, lx);
    const float hy = mdas_fma(p[6], wy, ly);
    const float cx = moving ? mdas_fma(p[4], t, p[0]) : p[0];
    const float cy = moving ? mdas_fma(p[5], t, p[1]) : p[1];
    const float dx = hx - cx;
    const float dy = hy - cy;
    return mdas_fma(dx, dx, dy * dy) <= p[7];
}

// Thin-lens camera at the origin looking down +z (SDK/cuda/whitted.cu:164-249):
// the pinhole ray through the film point meets the focal plane at
// focal * (nx * filmHalfW, ny * filmHalfH, 1); the lens ray starts at the lens
// sample and passes through that point.  All discs are fronto-parallel, so the
// nearest hit is the covering disc with the smallest depth (the first listed
// among equal depths).  Scenes keep their discs sorted by depth (stable), so
// the first covering disc in list order is that hit.
MDAS_HD void mdas_shade_discs_dof(const MdasScene* sc, const float* prims, const float* c, int moving,
                                  float* out) {
    float t, lx, ly, wx, wy;
    mdas_dof_ray(sc, c, moving, &t, &lx, &ly, &wx, &wy);
    float R = sc->background, G = sc->background, B = sc->background;
    for (int k = 0; k < sc->count; ++k) {
        const float* p = prims + MDAS_PRIM_STRIDE * k;
        if (mdas_disc_dof_covers(p, lx, ly, wx, wy, t, moving)) {
            R = p[8];
            G = p[9];
            B = p[10];
            break;
        }
    }
    out[0] = R;
    out[1] = G;
    out[2] = B;
}

// Ray-sphere test: nearest root t of |o + t d - c|^2 = r^2 with t in (tmin, tmax).
MDAS_HD float mdas_sphere_hit(const float* o, const float* d, const float* p, float tmin, float tmax) {
    const float oc[3] = {o[0] - p[0], o[1] - p[1], o[2] - p[2]};
    const float a = mdas_dot3(d, d);
    const float b = mdas_dot3(oc, d);
    const float cc = mdas_dot3(oc, oc) - p[7];
    const float disc = mdas_fma(b, b, -(a * cc));
    if (disc < 0.0f) return -1.0f;
    const float sq = sqrtf(disc);
    const float t0 = (-b - sq) / a;
    if (t0 > tmin && t0 < tmax) return t0;
    const float t1 = (-b + sq) / a;
    if (t1 > tmin && t1 < tmax) return t1;
    return -1.0f;
}

// Direct lighting with one light sample (SDK/cuda/direct.cu:116-152, 263-268):
// pinhole camera ray, nearest hit among the ground plane z = 0 and the spheres,
// light point = corner + (u, v) * size, analytic shadow ray against the spheres,
// Lambertian BRDF albedo/pi, radiance = brdf * E * A * cos_s * cos_l / dist^2.
MDAS_HD void mdas_shade_direct_light(const MdasScene* sc, const float* prims, const float* c, float* out) {
    const float px = c[0] / sc->scaleX;
    const float py = c[1] / sc->scaleY;
    const float nx = (px + px) - 1.0f;
    const float ny = (py + py) - 1.0f;
    float d[3];
    for (int i = 0; i < 3; ++i) d[i] = mdas_fma(nx, sc->U[i], mdas_fma(ny, sc->V[i], sc->W[i]));
    float tbest = 3.0e38f;
    int hit = -2;  // -2 nothing, -1 ground, k sphere k
    if (d[2] < 0.0f) {
        tbest = -sc->eye[2] / d[2];
        hit = -1;
    }
    for (int k = 0; k < sc->count; ++k) {
        const float t = mdas_sphere_hit(sc->eye, d, prims + MDAS_PRIM_STRIDE * k, 1.0e-4f, tbest);
        if (t > 0.0f) {
            tbest = t;
            hit = k;
        }
    }
    float L = sc->background;
    if (hit != -2) {
        float p[3], n[3];
        for (int i = 0; i < 3; ++i) p[i] = mdas_fma(tbest, d[i], sc->eye[i]);
        if (hit == -1) {
            n[0] = 0.0f;
            n[1] = 0.0f;
            n[2] = 1.0f;
        } else {
            const float* s = prims + MDAS_PRIM_STRIDE * hit;
            for (int i = 0; i < 3; ++i) n[i] = (p[i] - s[i]) * s[6];
        }
        const float u = c[2], v = c[3];
        const float q[3] = {mdas_fma(u, sc->lightSize, sc->lightCorner[0]),
                            mdas_fma(v, sc->lightSize, sc->lightCorner[1]), sc->lightCorner[2]};
        float po[3], wi[3];
        for (int i = 0; i < 3; ++i) {
            po[i] = mdas_fma(1.0e-3f, n[i], p[i]);
            wi[i] = q[i] - p[i];
        }
        const float d2 = mdas_dot3(wi, wi);
        const float invLen = 1.0f / sqrtf(d2);
        const float cosS = mdas_dot3(n, wi) * invLen;
        const float cosL = wi[2] * invLen;  // the light faces -z
        L = 0.0f;
        if (cosS > 0.0f && cosL > 0.0f) {
            const float seg[3] = {q[0] - po[0], q[1] - po[1], q[2] - po[2]};
            int blocked = 0;
            for (int k = 0; k < sc->count && !blocked; ++k)
                blocked = mdas_sphere_hit(po, seg, prims + MDAS_PRIM_STRIDE * k, 0.0f, 1.0f) > 0.0f;
            if (!blocked) {
                const float area = sc->lightSize * sc->lightSize;
                const float brdf = sc->albedo * 0.318309886f;  // 1/pi
                L = (((brdf * sc->emission) * area) * (cosS * cosL)) / d2;
            }
        }
    }
    out[0] = L;
    out[1] = L;
    out[2] = L;
}

MDAS_HD void mdas_shade(const MdasScene* sc, const float* prims, const float* c, float* out) {
    switch (sc->kind) {
        case MDAS_SCENE_DISCS_MB: mdas_shade_discs_mb(sc, prims, c, out); break;
        case MDAS_SCENE_DISCS_DOF: mdas_shade_discs_dof(sc, prims, c, 0, out); break;
        case MDAS_SCENE_DISCS_MBDOF: mdas_shade_discs_dof(sc, prims, c, 1, out); break;
        default: mdas_shade_direct_light(sc, prims, c, out); break;
    }
}
