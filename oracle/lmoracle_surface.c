/*
 * CPU oracle: surface geometry at triangle hits.
 *
 * TEST INFRASTRUCTURE ONLY (see lmoracle.h).  Restates, in double precision,
 * IntersectionUtils::CreateTriangleIntersection
 * (include/lightmetrica/intersectionutils.h:59-135) with the math it calls:
 *   hit point          p = o + d t, as an accel's Intersect forms it
 *                      (accel_naive.cpp:117-121)
 *   geometry normal    gn = Normalize(Cross(p2 - p1, p3 - p1))      :78-82
 *   shading normal     sn = Normalize(n1 (1 - b0 - b1) + n2 b0 + n3 b1), gn
 *                      when that is NaN or the mesh has no normals  :84-104
 *   texture coords     uv = uv1 (1 - b0 - b1) + uv2 b0 + uv3 b1, (0, 0)
 *                      without texcoords                            :106-115
 *   tangent frame      Math::OrthonormalBasis(sn, dpdu, dpdv)       :120-123,
 *                      math.h:2355-2359
 *   normal derivative  N = n1 (1 - b0 - b1) + n2 b0 + n3 b1,
 *                      dndu = (n2 - n1) / |N| - sn <., sn>,
 *                      dndv = (n3 - n2) / |N| - sn <., sn>          :125-131
 * Vector operations follow math.h's generic forms: Cross :1784-1787, Dot
 * :1721-1724, Normalize = v / Length(v) :1865-1868.  The per-triangle
 * vertices and normals are given already through the primitive's transform
 * and normal transform (intersectionutils.h:78-80, :91-93).
 */
#include "lmoracle.h"

#include <math.h>
#include <string.h>

typedef struct { double x, y, z; } v3;

static v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross(v3 a, v3 b)
{
    return mk(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static v3 normalize(v3 a)
{
    const double l = sqrt(dot(a, a));
    return mk(a.x / l, a.y / l, a.z / l);
}
static v3 at(const double* p, int k) { return mk(p[3 * k], p[3 * k + 1], p[3 * k + 2]); }
static double* put(double* o, v3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; return o + 3; }

void lmo_surface(const double* tris, const double* normals, const double* texcoords, const uint8_t* flags,
                 const double* rays, const double* hits, size_t n, double* out)
{
    for (size_t i = 0; i < n; i++) {
        double* o = out + 23 * i;
        const int prim = (int)hits[4 * i + 1];
        if (prim < 0) {
            memset(o, 0, 23 * sizeof(double));
            continue;
        }
        const double t = hits[4 * i], b0 = hits[4 * i + 2], b1 = hits[4 * i + 3];
        const double* r = rays + 8 * i;
        const v3 p = add(mk(r[0], r[1], r[2]), scl(mk(r[4], r[5], r[6]), t));
        const double* tv = tris + 9 * (size_t)prim;
        const v3 p1 = at(tv, 0), p2 = at(tv, 1), p3 = at(tv, 2);
        const v3 gn = normalize(cross(sub(p2, p1), sub(p3, p1)));
        const uint8_t fl = flags ? flags[prim] : (uint8_t)((normals ? 1 : 0) | (texcoords ? 2 : 0));
        const double w0 = 1.0 - b0 - b1;
        v3 n1 = gn, n2 = gn, n3 = gn, sn = gn;
        if ((fl & 1) && normals) {
            const double* nv = normals + 9 * (size_t)prim;
            n1 = at(nv, 0);
            n2 = at(nv, 1);
            n3 = at(nv, 2);
            sn = normalize(add(add(scl(n1, w0), scl(n2, b0)), scl(n3, b1)));
            if (isnan(sn.x) || isnan(sn.y) || isnan(sn.z)) sn = gn;
        }
        double u = 0.0, v = 0.0;
        if ((fl & 2) && texcoords) {
            const double* uv = texcoords + 6 * (size_t)prim;
            u = uv[0] * w0 + uv[2] * b0 + uv[4] * b1;
            v = uv[1] * w0 + uv[3] * b0 + uv[5] * b1;
        }
        const v3 dpdv = fabs(sn.x) > fabs(sn.y) ? normalize(mk(sn.z, 0.0, -sn.x)) : normalize(mk(0.0, sn.z, -sn.y));
        const v3 dpdu = cross(dpdv, sn);
        const v3 N = add(add(scl(n1, w0), scl(n2, b0)), scl(n3, b1));
        const double inv = 1.0 / sqrt(dot(N, N));
        const v3 dNdu = scl(sub(n2, n1), inv), dNdv = scl(sub(n3, n2), inv);
        const v3 dndu = sub(dNdu, scl(sn, dot(dNdu, sn)));
        const v3 dndv = sub(dNdv, scl(sn, dot(dNdv, sn)));
        o = put(o, p);
        o = put(o, gn);
        o = put(o, sn);
        o = put(o, dpdu);
        o = put(o, dpdv);
        o = put(o, dndu);
        o = put(o, dndv);
        o[0] = u;
        o[1] = v;
    }
}
