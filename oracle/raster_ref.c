/*
 * raster_ref.c -- CPU restatement of pybatchrender's render path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle and the timed CPU
 * baseline; the product renderer never links, loads or calls it.  Only tests/,
 * __graft_entry__.smoke() and bench.py (its cpu_baseline leg and the
 * "--impl reference" arm) use it.
 *
 * Built twice from this one source (see oracle/Makefile / oracle/build.py):
 *   REAL=double  -> symbols *_f64  (the FP64 parity reference)
 *   REAL=float   -> symbols *_f32  (the FP32 multithreaded CPU baseline)
 *
 * What it restates (paths relative to the reference project):
 *   shaders/basic.vert:24-57     instance decode (scene = gid / I, inst = gid % I,
 *                                id = shared ? inst : gid), clip = VP[scene] * M[id] * v,
 *                                v_normal = normalize(mat3(M) * n), v_color = colbuf[id]
 *   shaders/basic.frag:20-39     tile discard, base = 1 (useTexture = 0) or the
 *                                bilinear texture sample at the perspective-correct
 *                                v_uv (useTexture = 1: renderer/node.py:277-287),
 *                                ndl = max(dot(normalize(n), normalize(L)), 0),
 *                                l = mix(1, ambient + ndl * col, clamp(strength, 0, 1)),
 *                                rgb = base * color.rgb * l, a = color.a
 *   renderer/shader_context.py:47-84  R = Rz(H) Ry(P) Rx(R), M = [R*s | t]
 *   renderer/node.py:116-126     M[:3,:3] = rot3 * scale, M[:3,3] = position
 *   renderer/camera.py:110-135 + shaders/basic.vert:45-52
 *                                per-scene tile viewport; equivalent to rendering scene k
 *                                into its own W x H image with the GL viewport transform
 *   renderer/frame_grabber.py:105,167  vertical flip: image row 0 is the top row
 *   renderer/renderer.py:352-363 scene order of the [N,C,H,W] output
 *   renderer/renderer.py:262     clear colour (default black, alpha 1)
 *
 * The rasterisation rules are the GL contract the reference relies on through
 * the OpenGL driver (not in the reference sources; the driver's own choices
 * are not pinned by any reference test): pixel centres at +0.5, triangles
 * clipped against the near plane (z_clip >= -w_clip), back faces culled
 * (Panda3D's default cull mode: counter-clockwise front faces in GL window
 * coordinates), top-left fill rule, depth test strict-less against a 1.0
 * clear, equal depths resolved by draw order (node, then instance, then
 * triangle), window depth = 0.5 * z_ndc + 0.5, screen-linear depth and
 * perspective-correct normal interpolation, UNORM8 = floor(clamp(c,0,1)*255+0.5).
 * Textures follow GL's sampler defaults that Panda3D applies to a loaded
 * texture (linear min/mag filter without mipmaps, repeat wrap): texel
 * centres at (i + 0.5) / w, texel row 0 at v = 0 (the bottom row of the
 * image, Panda3D's image origin), RGBA8 texels read as c / 255.
 *
 * Pinning.  Everything before rasterisation (baked vertices, instance
 * matrices, colours, view-projection matrices, tiles, uniforms) is pinned by
 * fixtures recorded from the reference's own code (tests/golden/).  The raster
 * and shading rules are pinned by analytic known-answer tests
 * (tests/test_oracle_kat.py, tests/test_api_kat_cpu.py).  Pixel parity against
 * the reference's own renders is UNPINNED: the reference draws through
 * Panda3D/OpenGL, which cannot run on these machines, and it holds no pixel
 * fixture of its own.
 */
#include <math.h>
#include <tgmath.h> /* sin/cos/sqrt/exp follow REAL: float math in the FP32 build */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL double
#endif
#ifndef SFX
#define SFX _f64
#endif
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

typedef REAL real;

#define SOFT_CUTOFF 16.0  /* soft coverage is 0 beyond 16 sigma outside an edge */
#define SOFT_TAPER 4.0    /* tapered to 0 over the last 4 sigma */
#define SOFT_DEPTH_SAT 0.125 /* saturation depth of the extended plane, in units of zfar - znear */

#define ORC_MODE_HPR 0
#define ORC_MODE_ROT 1
#define ORC_MODE_MAT 2

typedef struct {
    int32_t nv, nt;
    const float* pos;    /* [nv*3] */
    const float* nrm;    /* [nv*3] */
    const int32_t* idx;  /* [nt*3] */
    const float* uv;     /* [nv*2] texture coordinates, or NULL (all 0) */
} orc_mesh;

typedef struct {
    int32_t mesh;
    int32_t inst_per_scene; /* I */
    int32_t shared;         /* 1: instance i of every scene reads buffer row i */
    int32_t mode;           /* ORC_MODE_* */
    const int32_t* counts;  /* [N] active instances per scene, or NULL (= I) */
    const float* pos;       /* [B*3] */
    const float* rot;       /* HPR [B*3] radians | ROT [B*9] | MAT [B*16] row-major */
    const float* scale;     /* [B] (ignored for MAT) */
    const float* color;     /* [B*4] */
    const uint8_t* tex;     /* [tex_h][tex_w][4] RGBA8, row 0 at v = 0; NULL: untextured */
    int32_t tex_w, tex_h;
} orc_node;

typedef struct {
    int32_t N, W, H, C;
    const float* vp;        /* [N*16] row-major view-projection per scene */
    float ambient[3], ldir[3], lcol[3], strength;
    float bg[4];
    int32_t cull;           /* 1: cull back faces (default) */
    /* soft mode */
    float znear, zfar, sigma, gamma;
    int32_t soft_dense;     /* unused (kept for layout) */
} orc_scene;

/* ------------------------------------------------------------------------ */

typedef struct {
    real m[12];             /* 3x4 row-major affine model matrix */
    real c[4];              /* colour */
} inst_xf;

static void build_instance(const orc_node* nd, int64_t id, inst_xf* out) {
    real R[9];
    const float* p = nd->pos + id * 3;
    if (nd->mode == ORC_MODE_MAT) {
        const float* mm = nd->rot + id * 16;
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) out->m[r * 4 + c] = (real)mm[r * 4 + c];
    } else {
        if (nd->mode == ORC_MODE_HPR) {
            const float* a = nd->rot + id * 3;
            real h = a[0], pp = a[1], rr = a[2];
            real ch = cos(h), sh = sin(h), cp = cos(pp), sp = sin(pp), cr = cos(rr), sr = sin(rr);
            /* Rz(H) @ Ry(P) @ Rx(R), renderer/shader_context.py:63-82 */
            R[0] = ch * cp; R[1] = ch * sp * sr - sh * cr; R[2] = ch * sp * cr + sh * sr;
            R[3] = sh * cp; R[4] = sh * sp * sr + ch * cr; R[5] = sh * sp * cr - ch * sr;
            R[6] = -sp;     R[7] = cp * sr;                R[8] = cp * cr;
        } else {
            const float* a = nd->rot + id * 9;
            for (int i = 0; i < 9; ++i) R[i] = a[i];
        }
        real s = nd->scale[id];
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) out->m[r * 4 + c] = R[r * 3 + c] * s;
            out->m[r * 4 + 3] = p[r];
        }
    }
    for (int i = 0; i < 4; ++i) out->c[i] = nd->color[id * 4 + i];
}

typedef struct {
    real x, y, z, w;        /* clip coordinates */
    real n[3];              /* world normal (normalised, basic.vert:53) */
    real u, v;              /* texture coordinates (basic.vert:56) */
} cvert;

static void xform_vertex(const inst_xf* xf, const real* VP, const float* p, const float* n, const float* uv,
                         cvert* o) {
    o->u = uv ? (real)uv[0] : 0;
    o->v = uv ? (real)uv[1] : 0;
    real wx = xf->m[0] * p[0] + xf->m[1] * p[1] + xf->m[2] * p[2] + xf->m[3];
    real wy = xf->m[4] * p[0] + xf->m[5] * p[1] + xf->m[6] * p[2] + xf->m[7];
    real wz = xf->m[8] * p[0] + xf->m[9] * p[1] + xf->m[10] * p[2] + xf->m[11];
    o->x = VP[0] * wx + VP[1] * wy + VP[2] * wz + VP[3];
    o->y = VP[4] * wx + VP[5] * wy + VP[6] * wz + VP[7];
    o->z = VP[8] * wx + VP[9] * wy + VP[10] * wz + VP[11];
    o->w = VP[12] * wx + VP[13] * wy + VP[14] * wz + VP[15];
    real nx = xf->m[0] * n[0] + xf->m[1] * n[1] + xf->m[2] * n[2];
    real ny = xf->m[4] * n[0] + xf->m[5] * n[1] + xf->m[6] * n[2];
    real nz = xf->m[8] * n[0] + xf->m[9] * n[1] + xf->m[10] * n[2];
    real ln = sqrt(nx * nx + ny * ny + nz * nz);
    real inv = ln > 0 ? (real)1 / ln : (real)0;
    o->n[0] = nx * inv; o->n[1] = ny * inv; o->n[2] = nz * inv;
}

/* Clip a triangle against the near plane z + w >= 0 (Sutherland-Hodgman).
 * Returns the vertex count of the clipped polygon (0, 3 or 4). */
static int clip_near(const cvert* in, cvert* out) {
    int n = 0;
    for (int i = 0; i < 3; ++i) {
        const cvert* a = &in[i];
        const cvert* b = &in[(i + 1) % 3];
        real da = a->z + a->w, db = b->z + b->w;
        if (da >= 0) out[n++] = *a;
        if ((da >= 0) != (db >= 0)) {
            real t = da / (da - db);
            cvert v;
            v.x = a->x + t * (b->x - a->x);
            v.y = a->y + t * (b->y - a->y);
            v.z = a->z + t * (b->z - a->z);
            v.w = a->w + t * (b->w - a->w);
            for (int k = 0; k < 3; ++k) v.n[k] = a->n[k] + t * (b->n[k] - a->n[k]);
            v.u = a->u + t * (b->u - a->u);
            v.v = a->v + t * (b->v - a->v);
            out[n++] = v;
        }
    }
    return n;
}

typedef struct {
    real sx[3], sy[3], sz[3], iw[3];   /* screen x, y (pixels, y down), window depth, 1/w */
    real n[3][3];
    real uv[3][2];
    const orc_node* tex_node;          /* node whose texture is sampled, or NULL */
    real A[3], B[3], Cc[3];            /* edge functions, edge k opposite vertex k */
    int tl[3];
    real area2;
    int x0, x1, y0, y1;                /* inclusive pixel bbox, clamped */
} stri;

/* Edge k runs from vertex (k+1)%3 to (k+2)%3; E_k(p) = A p.x + B p.y + C is
 * positive on the triangle's side and equals area2 * barycentric_k. */
static void setup_edges(stri* t) {
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        t->A[k] = t->sy[a] - t->sy[b];
        t->B[k] = t->sx[b] - t->sx[a];
        t->Cc[k] = -(t->A[k] * t->sx[a] + t->B[k] * t->sy[a]);
        /* top-left rule in image coordinates (y down) */
        t->tl[k] = (t->A[k] > 0) || (t->A[k] == 0 && t->B[k] > 0);
    }
}

/* Screen-space setup of one clipped triangle.  Returns 0 when it is culled.
 * margin: extra pixels around the image that still count (the soft mode's
 * coverage reaches pixels up to its cutoff distance outside the triangle). */
static int setup_tri(const orc_scene* sc, const cvert* v0, const cvert* v1, const cvert* v2, stri* t, real margin) {
    const cvert* v[3] = {v0, v1, v2};
    for (int k = 0; k < 3; ++k) {
        real iw = (real)1 / v[k]->w;
        t->sx[k] = (v[k]->x * iw + 1) * (real)0.5 * sc->W;
        t->sy[k] = (1 - v[k]->y * iw) * (real)0.5 * sc->H;
        t->sz[k] = v[k]->z * iw * (real)0.5 + (real)0.5;
        t->iw[k] = iw;
        for (int c = 0; c < 3; ++c) t->n[k][c] = v[k]->n[c];
        t->uv[k][0] = v[k]->u;
        t->uv[k][1] = v[k]->v;
    }
    t->tex_node = NULL;
    real area2 = (t->sx[1] - t->sx[0]) * (t->sy[2] - t->sy[0]) - (t->sx[2] - t->sx[0]) * (t->sy[1] - t->sy[0]);
    /* GL front faces are counter-clockwise with y up, i.e. area2 < 0 with y down */
    if (area2 == 0) return 0;
    if (area2 > 0) {
        if (sc->cull) return 0;
    }
    if (area2 < 0) {
        /* swap vertices 1 and 2 so that the interior is on the positive side */
        real tmp;
#define SWP(a, b) (tmp = (a), (a) = (b), (b) = tmp)
        SWP(t->sx[1], t->sx[2]); SWP(t->sy[1], t->sy[2]); SWP(t->sz[1], t->sz[2]); SWP(t->iw[1], t->iw[2]);
        for (int c = 0; c < 3; ++c) SWP(t->n[1][c], t->n[2][c]);
        SWP(t->uv[1][0], t->uv[2][0]); SWP(t->uv[1][1], t->uv[2][1]);
#undef SWP
        area2 = -area2;
    }
    t->area2 = area2;
    setup_edges(t);
    real mnx = t->sx[0], mxx = t->sx[0], mny = t->sy[0], mxy = t->sy[0];
    for (int k = 1; k < 3; ++k) {
        if (t->sx[k] < mnx) mnx = t->sx[k];
        if (t->sx[k] > mxx) mxx = t->sx[k];
        if (t->sy[k] < mny) mny = t->sy[k];
        if (t->sy[k] > mxy) mxy = t->sy[k];
    }
    /* pixels whose centre (x+0.5) can lie in [mn, mx], widened by one pixel */
    real fx0 = floor(mnx - (real)0.5 - margin) - 1, fx1 = ceil(mxx - (real)0.5 + margin) + 1;
    real fy0 = floor(mny - (real)0.5 - margin) - 1, fy1 = ceil(mxy - (real)0.5 + margin) + 1;
    if (fx1 < 0 || fy1 < 0 || fx0 > sc->W - 1 || fy0 > sc->H - 1) return 0;
    t->x0 = fx0 < 0 ? 0 : (int)fx0;
    t->y0 = fy0 < 0 ? 0 : (int)fy0;
    t->x1 = fx1 > sc->W - 1 ? sc->W - 1 : (int)fx1;
    t->y1 = fy1 > sc->H - 1 ? sc->H - 1 : (int)fy1;
    return 1;
}

static inline int covers(const stri* t, const real E[3]) {
    for (int k = 0; k < 3; ++k) {
        if (E[k] > 0) continue;
        if (E[k] == 0 && t->tl[k]) continue;
        return 0;
    }
    return 1;
}

static inline real clamp01(real v) { return v < 0 ? 0 : (v > 1 ? 1 : v); }

static inline uint8_t to_unorm8(real v) {
    return (uint8_t)floor(clamp01(v) * (real)255 + (real)0.5);
}

/* basic.frag:33-38 for a world normal n (not yet normalised). */
static void shade(const orc_scene* sc, const real Ln[3], const real n_in[3], const real col[4], real out[4]) {
    real ln = sqrt(n_in[0] * n_in[0] + n_in[1] * n_in[1] + n_in[2] * n_in[2]);
    real inv = ln > 0 ? (real)1 / ln : (real)0;
    real ndl = (n_in[0] * Ln[0] + n_in[1] * Ln[1] + n_in[2] * Ln[2]) * inv;
    if (!(ndl > 0)) ndl = 0;
    real s = clamp01((real)sc->strength);
    for (int c = 0; c < 3; ++c) {
        real light = (real)sc->ambient[c] + ndl * (real)sc->lcol[c];
        real l = (real)1 * (1 - s) + light * s;
        out[c] = col[c] * l;
    }
    out[3] = col[3];
}

/* GL bilinear sample with repeat wrap of an RGBA8 texture (row 0 at v = 0). */
static void sample_texture(const orc_node* nd, real u, real v, real out[3]) {
    const int w = nd->tex_w, h = nd->tex_h;
    real fu = u - floor(u), fv = v - floor(v);
    real x = fu * w - (real)0.5, y = fv * h - (real)0.5;
    real fx = floor(x), fy = floor(y);
    real ax = x - fx, ay = y - fy;
    /* fx lies in [-1, w - 1]; -1 wraps to w - 1 (so does a NaN coordinate) */
    int x0 = (fx >= 0 && fx <= w - 1) ? (int)fx : w - 1;
    int y0 = (fy >= 0 && fy <= h - 1) ? (int)fy : h - 1;
    int x1 = x0 + 1 == w ? 0 : x0 + 1, y1 = y0 + 1 == h ? 0 : y0 + 1;
    const uint8_t* t00 = nd->tex + ((int64_t)y0 * w + x0) * 4;
    const uint8_t* t10 = nd->tex + ((int64_t)y0 * w + x1) * 4;
    const uint8_t* t01 = nd->tex + ((int64_t)y1 * w + x0) * 4;
    const uint8_t* t11 = nd->tex + ((int64_t)y1 * w + x1) * 4;
    for (int c = 0; c < 3; ++c) {
        real top = (1 - ax) * (t00[c] / (real)255) + ax * (t10[c] / (real)255);
        real bot = (1 - ax) * (t01[c] / (real)255) + ax * (t11[c] / (real)255);
        out[c] = (1 - ay) * top + ay * bot;
    }
}

static void light_dir(const orc_scene* sc, real Ln[3]) {
    real lx = sc->ldir[0], ly = sc->ldir[1], lz = sc->ldir[2];
    real ln = sqrt(lx * lx + ly * ly + lz * lz);
    real inv = ln > 0 ? (real)1 / ln : (real)0;
    Ln[0] = lx * inv; Ln[1] = ly * inv; Ln[2] = lz * inv;
}

/* Walk every triangle of scene k in draw order.  The callback receives the
 * screen triangle, its instance colour and its winner id. */
typedef void (*tri_cb)(void* user, const stri* t, const real col[4], int32_t wid);

static int scene_max_tris(int nmeshes, const orc_mesh* meshes) {
    int mt = 1;
    for (int i = 0; i < nmeshes; ++i)
        if (meshes[i].nt > mt) mt = meshes[i].nt;
    return mt;
}

static void walk_scene(const orc_scene* sc, int nmeshes, const orc_mesh* meshes, int nnodes,
                       const orc_node* nodes, int k, int soft, tri_cb cb, void* user) {
    real VP[16];
    for (int i = 0; i < 16; ++i) VP[i] = sc->vp[(int64_t)k * 16 + i];
    int max_tris = scene_max_tris(nmeshes, meshes);
    int rank_base = 0;
    cvert* cache = NULL;
    int cache_cap = 0;
    for (int n = 0; n < nnodes; ++n) {
        const orc_node* nd = &nodes[n];
        const orc_mesh* me = &meshes[nd->mesh];
        int ips = nd->inst_per_scene;
        int cnt = nd->counts ? nd->counts[k] : ips;
        if (cnt > ips) cnt = ips;
        if (me->nv > cache_cap) {
            free(cache);
            cache_cap = me->nv;
            cache = (cvert*)malloc(sizeof(cvert) * (size_t)cache_cap);
        }
        for (int i = 0; i < cnt; ++i) {
            int64_t id = nd->shared ? (int64_t)i : (int64_t)k * ips + i;
            inst_xf xf;
            build_instance(nd, id, &xf);
            for (int v = 0; v < me->nv; ++v)
                xform_vertex(&xf, VP, me->pos + 3 * v, me->nrm + 3 * v, me->uv ? me->uv + 2 * v : NULL, &cache[v]);
            int32_t wid_base = (int32_t)((rank_base + i) * max_tris);
            for (int t = 0; t < me->nt; ++t) {
                cvert tv[3];
                for (int c = 0; c < 3; ++c) tv[c] = cache[me->idx[3 * t + c]];
                cvert poly[4];
                int np;
                if (soft) {
                    /* soft mode drops triangles that are not fully in front of the near plane */
                    if (tv[0].z + tv[0].w < 0 || tv[1].z + tv[1].w < 0 || tv[2].z + tv[2].w < 0) continue;
                    for (int c = 0; c < 3; ++c) poly[c] = tv[c];
                    np = 3;
                } else {
                    np = clip_near(tv, poly);
                }
                for (int f = 1; f + 1 < np; ++f) {
                    stri st;
                    real margin = soft ? (real)SOFT_CUTOFF * (real)sc->sigma + 1 : 0;
                    if (!setup_tri(sc, &poly[0], &poly[f], &poly[f + 1], &st, margin)) continue;
                    st.tex_node = nd->tex ? nd : NULL;
                    cb(user, &st, xf.c, wid_base + t);
                }
            }
        }
        rank_base += ips;
    }
    free(cache);
}

/* ------------------------------------------------------------------------ */
/* Hard raster                                                               */

typedef struct {
    const orc_scene* sc;
    real Ln[3];
    real* zbuf;       /* [H*W] */
    real* rgba;       /* [H*W*4] */
    int32_t* win;     /* [H*W] */
    uint8_t* amb;     /* [H*W] or NULL */
    real tol_px, tol_z;
} hard_ctx;

static void hard_pass1(void* user, const stri* t, const real col[4], int32_t wid) {
    hard_ctx* h = (hard_ctx*)user;
    const orc_scene* sc = h->sc;
    for (int y = t->y0; y <= t->y1; ++y) {
        real py = y + (real)0.5;
        for (int x = t->x0; x <= t->x1; ++x) {
            real px = x + (real)0.5;
            real E[3];
            for (int k = 0; k < 3; ++k) E[k] = t->A[k] * px + t->B[k] * py + t->Cc[k];
            if (!covers(t, E)) continue;
            real b0 = E[0] / t->area2, b1 = E[1] / t->area2, b2 = E[2] / t->area2;
            real z = b0 * t->sz[0] + b1 * t->sz[1] + b2 * t->sz[2];
            if (z < 0) z = 0; /* GL clamps window depth to [0,1] */
            int64_t o = (int64_t)y * sc->W + x;
            if (!(z < h->zbuf[o])) continue;
            h->zbuf[o] = z;
            h->win[o] = wid;
            /* perspective-correct normal (basic.frag:33) */
            real q0 = b0 * t->iw[0], q1 = b1 * t->iw[1], q2 = b2 * t->iw[2];
            real qs = q0 + q1 + q2;
            real nn[3];
            for (int c = 0; c < 3; ++c) nn[c] = (q0 * t->n[0][c] + q1 * t->n[1][c] + q2 * t->n[2][c]) / qs;
            if (t->tex_node) {
                /* basic.frag:31-32,38: base * v_color.rgb */
                real u = (q0 * t->uv[0][0] + q1 * t->uv[1][0] + q2 * t->uv[2][0]) / qs;
                real v = (q0 * t->uv[0][1] + q1 * t->uv[1][1] + q2 * t->uv[2][1]) / qs;
                real base[3], tc[4];
                sample_texture(t->tex_node, u, v, base);
                for (int c = 0; c < 3; ++c) tc[c] = base[c] * col[c];
                tc[3] = col[3];
                shade(sc, h->Ln, nn, tc, &h->rgba[o * 4]);
            } else {
                shade(sc, h->Ln, nn, col, &h->rgba[o * 4]);
            }
        }
    }
}

/* Second walk: flag pixels whose centre lies within tol_px of an edge of a
 * triangle that is (nearly) visible there, or that another covering
 * fragment ties in depth within tol_z. */
static void hard_pass2(void* user, const stri* t, const real col[4], int32_t wid) {
    (void)col;
    hard_ctx* h = (hard_ctx*)user;
    const orc_scene* sc = h->sc;
    real L[3];
    for (int k = 0; k < 3; ++k) L[k] = sqrt(t->A[k] * t->A[k] + t->B[k] * t->B[k]);
    for (int y = t->y0; y <= t->y1; ++y) {
        real py = y + (real)0.5;
        for (int x = t->x0; x <= t->x1; ++x) {
            real px = x + (real)0.5;
            real E[3], dmin = 1e30;
            for (int k = 0; k < 3; ++k) {
                E[k] = t->A[k] * px + t->B[k] * py + t->Cc[k];
                real d = L[k] > 0 ? E[k] / L[k] : 0;
                if (d < dmin) dmin = d;
            }
            real b0 = E[0] / t->area2, b1 = E[1] / t->area2, b2 = E[2] / t->area2;
            real z = b0 * t->sz[0] + b1 * t->sz[1] + b2 * t->sz[2];
            if (z < 0) z = 0;
            int64_t o = (int64_t)y * sc->W + x;
            real zb = h->zbuf[o];
            if (fabs(dmin) < h->tol_px && z <= zb + h->tol_z && z < 1) h->amb[o] = 1;
            if (covers(t, E) && h->win[o] != wid && fabs(z - zb) < h->tol_z) h->amb[o] = 1;
        }
    }
}

typedef struct {
    const orc_scene* sc;
    int nmeshes;
    const orc_mesh* meshes;
    int nnodes;
    const orc_node* nodes;
    uint8_t* out;
    float* depth;
    int32_t* winner;
    uint8_t* ambiguous;
    real tol_px, tol_z;
    int k0, k1;
    int status;
} hard_job;

static void* hard_worker(void* arg) {
    hard_job* j = (hard_job*)arg;
    const orc_scene* sc = j->sc;
    int64_t P = (int64_t)sc->W * sc->H;
    hard_ctx h;
    h.sc = sc;
    light_dir(sc, h.Ln);
    h.zbuf = (real*)malloc(sizeof(real) * P);
    h.rgba = (real*)malloc(sizeof(real) * P * 4);
    h.win = (int32_t*)malloc(sizeof(int32_t) * P);
    h.amb = j->ambiguous ? (uint8_t*)malloc((size_t)P) : NULL;
    h.tol_px = j->tol_px;
    h.tol_z = j->tol_z;
    if (!h.zbuf || !h.rgba || !h.win || (j->ambiguous && !h.amb)) {
        j->status = -1;
        free(h.zbuf); free(h.rgba); free(h.win); free(h.amb);
        return NULL;
    }
    for (int k = j->k0; k < j->k1; ++k) {
        for (int64_t o = 0; o < P; ++o) {
            h.zbuf[o] = 1;
            h.win[o] = -1;
            for (int c = 0; c < 4; ++c) h.rgba[o * 4 + c] = sc->bg[c];
        }
        walk_scene(sc, j->nmeshes, j->meshes, j->nnodes, j->nodes, k, 0, hard_pass1, &h);
        if (h.amb) {
            memset(h.amb, 0, (size_t)P);
            walk_scene(sc, j->nmeshes, j->meshes, j->nnodes, j->nodes, k, 0, hard_pass2, &h);
            memcpy(j->ambiguous + (int64_t)k * P, h.amb, (size_t)P);
        }
        for (int c = 0; c < sc->C; ++c) {
            uint8_t* dst = j->out + ((int64_t)k * sc->C + c) * P;
            for (int64_t o = 0; o < P; ++o) dst[o] = to_unorm8(h.rgba[o * 4 + c]);
        }
        if (j->depth)
            for (int64_t o = 0; o < P; ++o) j->depth[(int64_t)k * P + o] = (float)h.zbuf[o];
        if (j->winner) memcpy(j->winner + (int64_t)k * P, h.win, sizeof(int32_t) * P);
    }
    free(h.zbuf); free(h.rgba); free(h.win); free(h.amb);
    return NULL;
}

/* Render scenes [k0, k1) into out[N,C,H,W] (scene-indexed; only the rows of
 * the requested scenes are written).  depth [N,H,W], winner [N,H,W] and
 * ambiguous [N,H,W] may be NULL.  Winner id = instance rank within the scene
 * (node-major) * max_triangles + triangle index, -1 for background. */
int FN(orc_render_hard)(const orc_scene* sc, int nmeshes, const orc_mesh* meshes, int nnodes,
                        const orc_node* nodes, int k0, int k1, uint8_t* out, float* depth,
                        int32_t* winner, uint8_t* ambiguous, float tol_px, float tol_z,
                        int nthreads) {
    if (!sc || !out || sc->W <= 0 || sc->H <= 0 || sc->C < 1 || sc->C > 4) return -2;
    if (k0 < 0 || k1 > sc->N || k0 > k1) return -2;
    if (nthreads < 1) nthreads = 1;
    int nscenes = k1 - k0;
    if (nthreads > nscenes) nthreads = nscenes > 0 ? nscenes : 1;
    hard_job* jobs = (hard_job*)calloc((size_t)nthreads, sizeof(hard_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int i = 0; i < nthreads; ++i) {
        hard_job* j = &jobs[i];
        j->sc = sc; j->nmeshes = nmeshes; j->meshes = meshes; j->nnodes = nnodes; j->nodes = nodes;
        j->out = out; j->depth = depth; j->winner = winner; j->ambiguous = ambiguous;
        j->tol_px = tol_px; j->tol_z = tol_z;
        j->k0 = k0 + (int)((int64_t)nscenes * i / nthreads);
        j->k1 = k0 + (int)((int64_t)nscenes * (i + 1) / nthreads);
    }
    int rc = 0;
    if (nthreads == 1) {
        hard_worker(&jobs[0]);
    } else {
        for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, hard_worker, &jobs[i]);
        for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    }
    for (int i = 0; i < nthreads; ++i)
        if (jobs[i].status) rc = jobs[i].status;
    free(jobs);
    free(th);
    return rc;
}

/* Model matrices as the renderer builds them: out [B,16] row-major 4x4. */
int FN(orc_instance_matrices)(const orc_node* nd, int64_t B, float* out) {
    for (int64_t id = 0; id < B; ++id) {
        inst_xf xf;
        build_instance(nd, id, &xf);
        for (int i = 0; i < 12; ++i) out[id * 16 + i] = (float)xf.m[i];
        out[id * 16 + 12] = 0; out[id * 16 + 13] = 0; out[id * 16 + 14] = 0; out[id * 16 + 15] = 1;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Soft coverage (differentiable mode)                                       */
/*
 * Per fragment (pixel p, front-facing triangle j fully in front of the near plane):
 *   e_k   = E_k(p) / |(A_k, B_k)|              signed distance to edge line k (px)
 *   D_j   = prod_k sigmoid(e_k / sigma) * T(d)   soft coverage; d = Euclidean distance
 *           from p to the triangle (0 inside), T(d) = S((16 sigma - d) / (4 sigma)),
 *           S(x) = x^3 (6x^2 - 15x + 10) on [0,1], 0 below, 1 above: exactly 0 once
 *           p is 16 sigma or more away from the triangle
 *   1/x   = sum_k b_k / w_k                    b_k = E_k / area2 (unclamped): the depth x
 *           of the triangle's plane; w = x up to w_hi = max_k w_k, w = w_hi + s (1 - exp(-(x -
 *           w_hi) / s)) beyond it with s = (zfar - znear) / 8, and w = w_hi + s where
 *           sum_k b_k / w_k <= 0: the extended plane's depth stays bounded and smooth instead of
 *           running off to infinity near the vanishing line of a face seen nearly edge-on
 *   zs_j  = (zfar - w) / (zfar - znear)        normalised linear depth, nearer = larger
 *   C_j   = basic.frag shading with the perspective-correct (extrapolated) normal,
 *           unclamped
 *   w_j   = D_j exp((zs_j - max zs) / gamma)
 *   A     = 1 - prod_j (1 - D_j)
 *   out   = A * sum_j w_j C_j / sum_j w_j + (1 - A) * bg.rgb
 */

/* smootherstep taper of the coverage tail, as a function of the distance d
 * from the pixel to the triangle */
static inline real soft_taper(real d, real sig) {
    real x = ((real)SOFT_CUTOFF * sig - d) / ((real)SOFT_TAPER * sig);
    if (x <= 0) return 0;
    if (x >= 1) return 1;
    return x * x * x * (x * (x * 6 - 15) + 10);
}

/* distance from (px,py) to the segment (ax,ay)-(bx,by) */
static inline real seg_dist(real px, real py, real ax, real ay, real bx, real by) {
    real ux = bx - ax, uy = by - ay, wx = px - ax, wy = py - ay;
    real l2 = ux * ux + uy * uy;
    real t = l2 > 0 ? (wx * ux + wy * uy) / l2 : 0;
    if (t < 0) t = 0;
    if (t > 1) t = 1;
    real dx = px - (ax + t * ux), dy = py - (ay + t * uy);
    return sqrt(dx * dx + dy * dy);
}

typedef struct {
    const orc_scene* sc;
    real Ln[3];
    real* m;      /* running max zs  [P] */
    real* S;      /* sum of weights  [P] */
    real* acc;    /* weighted colour [P*3] */
    real* Pi;     /* prod (1 - D)    [P] */
} soft_ctx;



static void soft_cb(void* user, const stri* t, const real col[4], int32_t wid) {
    (void)wid;
    soft_ctx* s = (soft_ctx*)user;
    const orc_scene* sc = s->sc;
    real sig = sc->sigma;
    real L[3];
    for (int k = 0; k < 3; ++k) L[k] = sqrt(t->A[k] * t->A[k] + t->B[k] * t->B[k]);
    int x0, x1, y0, y1;
    {
        /* bbox widened by the cutoff distance */
        real mnx = t->sx[0], mxx = t->sx[0], mny = t->sy[0], mxy = t->sy[0];
        for (int k = 1; k < 3; ++k) {
            if (t->sx[k] < mnx) mnx = t->sx[k];
            if (t->sx[k] > mxx) mxx = t->sx[k];
            if (t->sy[k] < mny) mny = t->sy[k];
            if (t->sy[k] > mxy) mxy = t->sy[k];
        }
        real r = SOFT_CUTOFF * sig + 1;
        real fx0 = floor(mnx - r), fx1 = ceil(mxx + r), fy0 = floor(mny - r), fy1 = ceil(mxy + r);
        if (fx1 < 0 || fy1 < 0 || fx0 > sc->W - 1 || fy0 > sc->H - 1) return;
        x0 = fx0 < 0 ? 0 : (int)fx0;
        y0 = fy0 < 0 ? 0 : (int)fy0;
        x1 = fx1 > sc->W - 1 ? sc->W - 1 : (int)fx1;
        y1 = fy1 > sc->H - 1 ? sc->H - 1 : (int)fy1;
    }
    for (int y = y0; y <= y1; ++y) {
        real py = y + (real)0.5;
        for (int x = x0; x <= x1; ++x) {
            real px = x + (real)0.5;
            real E[3], e[3], emin = 1e30;
            for (int k = 0; k < 3; ++k) {
                E[k] = t->A[k] * px + t->B[k] * py + t->Cc[k];
                e[k] = E[k] / L[k];
                if (e[k] < emin) emin = e[k];
            }
            if (emin <= -SOFT_CUTOFF * sig) continue;
            real dout = 0;
            if (emin < 0) {
                dout = 1e30;
                for (int k = 0; k < 3; ++k) {
                    int a = (k + 1) % 3, b = (k + 2) % 3;
                    real d = seg_dist(px, py, t->sx[a], t->sy[a], t->sx[b], t->sy[b]);
                    if (d < dout) dout = d;
                }
            }
            real D = soft_taper(dout, sig);
            for (int k = 0; k < 3; ++k) D *= (real)1 / (1 + exp(-e[k] / sig));
            if (!(D > 0)) continue;
            real b0 = E[0] / t->area2, b1 = E[1] / t->area2, b2 = E[2] / t->area2;
            real q0 = b0 * t->iw[0], q1 = b1 * t->iw[1], q2 = b2 * t->iw[2];
            real qs = q0 + q1 + q2;
            real whi = (real)1 / t->iw[0];
            for (int k = 1; k < 3; ++k) {
                real wk = (real)1 / t->iw[k];
                if (wk > whi) whi = wk;
            }
            real sat = (real)SOFT_DEPTH_SAT * ((real)sc->zfar - (real)sc->znear);
            real w = whi + sat;
            if (qs > 0) {
                w = (real)1 / qs;
                if (w > whi) w = whi + sat * (1 - exp(-(w - whi) / sat));
            }
            real zs = ((real)sc->zfar - w) / ((real)sc->zfar - (real)sc->znear);
            real nn[3], C[4];
            /* perspective-correct normal, oriented by the sign of the interpolation denominator */
            real orient = qs < 0 ? (real)-1 : (real)1;
            for (int c = 0; c < 3; ++c) nn[c] = (q0 * t->n[0][c] + q1 * t->n[1][c] + q2 * t->n[2][c]) * orient;
            shade(sc, s->Ln, nn, col, C);
            int64_t o = (int64_t)y * sc->W + x;
            s->Pi[o] *= (1 - D);
            if (zs > s->m[o]) {
                real f = exp((s->m[o] - zs) / (real)sc->gamma);
                s->S[o] = s->S[o] * f + D;
                for (int c = 0; c < 3; ++c) s->acc[o * 3 + c] = s->acc[o * 3 + c] * f + D * C[c];
                s->m[o] = zs;
            } else {
                real f = D * exp((zs - s->m[o]) / (real)sc->gamma);
                s->S[o] += f;
                for (int c = 0; c < 3; ++c) s->acc[o * 3 + c] += f * C[c];
            }
        }
    }
}

/* Soft render of scenes [k0,k1) into out[N,3,H,W]: float, or double when
 * out_double != 0 (finite-difference checks need the unrounded image). */
int FN(orc_render_soft)(const orc_scene* sc, int nmeshes, const orc_mesh* meshes, int nnodes,
                        const orc_node* nodes, int k0, int k1, void* out, int out_double) {
    if (!sc || !out || k0 < 0 || k1 > sc->N || k0 > k1) return -2;
    int64_t P = (int64_t)sc->W * sc->H;
    soft_ctx s;
    s.sc = sc;
    light_dir(sc, s.Ln);
    s.m = (real*)malloc(sizeof(real) * P);
    s.S = (real*)malloc(sizeof(real) * P);
    s.acc = (real*)malloc(sizeof(real) * P * 3);
    s.Pi = (real*)malloc(sizeof(real) * P);
    if (!s.m || !s.S || !s.acc || !s.Pi) {
        free(s.m); free(s.S); free(s.acc); free(s.Pi);
        return -1;
    }
    for (int k = k0; k < k1; ++k) {
        for (int64_t o = 0; o < P; ++o) {
            s.m[o] = -1e30; s.S[o] = 0; s.Pi[o] = 1;
            s.acc[o * 3] = s.acc[o * 3 + 1] = s.acc[o * 3 + 2] = 0;
        }
        walk_scene(sc, nmeshes, meshes, nnodes, nodes, k, 1, soft_cb, &s);
        for (int c = 0; c < 3; ++c) {
            for (int64_t o = 0; o < P; ++o) {
                real A = 1 - s.Pi[o];
                real fg = s.S[o] > 0 ? s.acc[o * 3 + c] / s.S[o] : 0;
                real v = A * fg + (1 - A) * (real)sc->bg[c];
                int64_t idx = ((int64_t)k * 3 + c) * P + o;
                if (out_double) ((double*)out)[idx] = (double)v;
                else ((float*)out)[idx] = (float)v;
            }
        }
    }
    free(s.m); free(s.S); free(s.acc); free(s.Pi);
    return 0;
}
