/*
 * pbr_capi.h -- C ABI of libpbr.so, the GB300 (sm_103a) batch renderer.
 *
 * The reference renders through Panda3D + OpenGL: per-instance matrices and
 * colours live in buffer textures uploaded with Texture.set_ram_image
 * (renderer/node.py:85-91,110-114,156-161), per-scene view-projection matrices
 * and tile rectangles in two more buffer textures (renderer/camera.py:29-30,
 * 110-135,146-148), lighting in shader uniforms (renderer/light.py:26-44),
 * one instanced draw per node runs shaders/basic.{vert,frag}, and the atlas is
 * read back and rearranged into [N,C,H,W] (renderer/renderer.py:326-363,
 * renderer/frame_grabber.py:85-106).  This ABI replaces that whole layer:
 * the caller keeps the scene state in device buffers it owns, binds their
 * addresses once, and every render call writes the final [N,C,H,W] pixels
 * directly into a caller-owned device tensor.
 *
 * Conventions
 *  - Every entry point returns an int status: PBR_OK (0) or a PBR_ERR_* code.
 *    pbr_last_error() returns a message for the last failing call on a context
 *    (or, with ctx == NULL, for the last failing pbr_create, or call given a
 *    null context, on this thread).  pbr_cartpole_step and pbr_camera_update
 *    take no context and report through their status alone.
 *  - Pointers named d_* are device pointers on the context's device.  They are
 *    borrowed, never freed: the caller keeps them alive while they are bound.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default
 *    stream.  Render/backward calls only enqueue kernels and asynchronous
 *    memsets on that stream: no host synchronisation and no allocation, so
 *    they may be captured into a CUDA graph.  Binding calls change kernel
 *    arguments; a graph captured before a rebind keeps the old arguments.
 *  - One context belongs to one host thread at a time.
 */
#ifndef PBR_CAPI_H
#define PBR_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pbr_ctx pbr_ctx;

#define PBR_OK 0
#define PBR_ERR_INVALID 1   /* bad argument (shape, pointer, range) */
#define PBR_ERR_CUDA 2      /* a CUDA runtime call failed */
#define PBR_ERR_CAPACITY 3  /* a fixed table or id range is exceeded */
#define PBR_ERR_STATE 4     /* call order (e.g. render before a camera is bound) */
#define PBR_ERR_DEVICE 5    /* a kernel reported an error flag (see pbr_device_status) */

/* Instance rotation encodings for pbr_node_set_buffers(mode). */
#define PBR_MODE_HPR 0  /* d_rot = [B,3] heading/pitch/roll in radians, R = Rz(H) Ry(P) Rx(R) */
#define PBR_MODE_ROT 1  /* d_rot = [B,9] row-major 3x3 rotation */
#define PBR_MODE_MAT 2  /* d_rot = [B,16] row-major 4x4 model matrix; d_pos, d_scale unused */

/* Library version (major*10000 + minor*100 + patch).  No counterpart in the
 * reference. */
int pbr_version(void);

/* Message for the last failing call.  Never NULL. */
const char* pbr_last_error(const pbr_ctx* ctx);

/* Create a renderer for num_scenes scenes of width x height pixels with
 * `channels` output channels (1..4: R, G, B, A).  Replaces the window/atlas
 * set-up of PBRRenderer.__init__ + _setup_offscreen_rt
 * (renderer/renderer.py:39-89,253-287) and PBRConfig.process_resolution
 * (config.py:61-126): scenes are a flat batch, there is no atlas.
 * flags: reserved, pass 0. */
int pbr_create(pbr_ctx** out_ctx, int num_scenes, int width, int height, int channels, int flags);
int pbr_destroy(pbr_ctx* ctx);

/* Register a triangle mesh already resident on the device: d_pos [nv,3],
 * d_nrm [nv,3] (unit normals), d_idx [nt,3] counter-clockwise seen from
 * outside.  smooth = 0 when every triangle's three normals are equal (flat
 * shading is then resolved once per triangle).  Replaces the model load +
 * flattenStrong of PBRNode.__init__ (renderer/node.py:61-71). */
int pbr_mesh_register(pbr_ctx* ctx, const float* d_pos, const float* d_nrm, const int32_t* d_idx,
                      int nv, int nt, int smooth, int* out_mesh_id);

/* Bounding sphere of a registered mesh (centre and radius in mesh
 * coordinates, every vertex within it).  With it the tile kernel skips the
 * instances whose bound projects outside the pixel region it is drawing.
 * Optional (radius 0: no skipping); no counterpart in the reference. */
int pbr_mesh_set_bounds(pbr_ctx* ctx, int mesh_id, float cx, float cy, float cz, float radius);

/* Optional: clusters of 32 consecutive triangles of a mesh, so that the tile
 * kernel can skip groups of triangles before setting them up: d_clusters
 * [num_clusters, 8] float32, 16-byte aligned, num_clusters = ceil(nt / 32);
 * per cluster its bounding sphere (cx, cy, cz, r) in mesh coordinates and the
 * cone of its triangles' geometric normals (unit axis ax, ay, az and the
 * cosine of the cone's half-angle; <= 0: no cone).  A cluster is skipped when
 * all its triangles face away from the eye (HPR poses) or its projected sphere
 * holds no pixel centre of the region drawn; the pixels are the same as without
 * clusters.  NULL removes them.  No reference counterpart (Panda3D draws every
 * triangle). */
int pbr_mesh_set_clusters(pbr_ctx* ctx, int mesh_id, const float* d_clusters, int num_clusters,
                          int cluster_triangles);

/* Attach texture coordinates to a registered mesh: d_uv [nv,2] float32
 * (GL convention, v = 0 at the bottom of the image), or NULL for none (all
 * coordinates 0).  Replaces the p3d_MultiTexCoord0 vertex column that
 * Panda3D's model loader provides (renderer/node.py:61-71,
 * shaders/basic.vert:16,56). */
int pbr_mesh_set_uv(pbr_ctx* ctx, int mesh_id, const float* d_uv);

/* Add a node: one mesh drawn instances_per_scene times in every scene.
 * shared != 0 means instance i of every scene reads buffer row i
 * (B = instances_per_scene rows), otherwise scene k instance i reads row
 * k*instances_per_scene + i (B = N*instances_per_scene rows).  Replaces
 * PBRNode's instance count and the instancesPerScene / shareAcrossScenes
 * uniforms (renderer/node.py:43-46,68,90-91; shaders/basic.vert:25-28).
 * Nodes draw in the order they are added (the reference's draw order). */
int pbr_node_add(pbr_ctx* ctx, int mesh_id, int instances_per_scene, int shared, int* out_node_id);

/* Bind a node's per-instance device buffers (float32, B rows):
 * d_pos [B,3], d_rot (see PBR_MODE_*), d_scale [B], d_color [B,4] RGBA.
 * d_counts [N] int32 (optional, may be NULL): active instances of this node
 * in scene k (0..instances_per_scene).  Replaces matbuf/colbuf uploads
 * (renderer/node.py:110-178): the kernels build M = [R*s | t] themselves. */
int pbr_node_set_buffers(pbr_ctx* ctx, int node_id, int mode, const float* d_pos, const float* d_rot,
                         const float* d_scale, const float* d_color, const int32_t* d_counts);

/* Texture a node (useTexture = 1): d_rgba [height,width,4] uint8 RGBA on the
 * device, row 0 at v = 0 (the bottom row of the image, Panda3D's image
 * origin), 4-byte aligned; NULL removes the texture (useTexture = 0).
 * Sampled per pixel with bilinear filtering and repeat wrap at the
 * perspective-correct texture coordinates; the shaded colour becomes
 * texel.rgb * colour.rgb * light.  Hard raster only: the soft-mode calls
 * fail with PBR_ERR_INVALID while a node is textured.  Replaces
 * PBRNode.set_texture (renderer/node.py:277-287) and the p3d_Texture0 sample
 * of shaders/basic.frag:31-32. */
int pbr_node_set_texture(pbr_ctx* ctx, int node_id, const uint8_t* d_rgba, int width, int height);

/* Bind pose component `component` of a node to column `column` of a per-step
 * state matrix: 0..2 = position x, y, z; 3..5 = heading, pitch, roll (HPR
 * mode).  column < 0 removes the binding.  Buffer row r of the node reads
 * state row r (scene k, instance i of a per-scene node: row
 * k*instances_per_scene + i).  The bound values are used by
 * pbr_render_state only.  Replaces an env's _step() that copies state
 * columns into node poses (envs/cartpole/renderer.py:98-140 copies cart x,
 * pole x and pole pitch): the copy happens inside the raster launch. */
int pbr_node_bind_state(pbr_ctx* ctx, int node_id, int component, int column);

/* Set (d_state non-NULL) or clear (NULL) the state matrix the bound pose
 * components read: float32, `rows` rows of `cols` values, row r at
 * d_state + r*row_stride.  Checked against every binding (column < cols,
 * enough rows, angles only on HPR-mode nodes). */
int pbr_state_source(pbr_ctx* ctx, const float* d_state, long long rows, int cols, long long row_stride);

/* Bind the per-scene view-projection matrices d_vp [N,16] (row-major, GL
 * clip-space conventions) and the camera's near/far planes (used by the soft
 * mode's depth normalisation).  Replaces viewbuf (renderer/camera.py:146-148,
 * 252-262) and tilebuf (camera.py:110-135): scene k renders into its own
 * W x H image, which is what the tile viewport of shaders/basic.vert:45-52
 * plus the discard of shaders/basic.frag:22-29 amount to. */
int pbr_camera_bind(pbr_ctx* ctx, const float* d_vp, float z_near, float z_far);

/* Lighting uniforms of shaders/basic.frag:13-18 (renderer/light.py:26-44):
 * ambient colour, direction *towards* the light (normalised by the kernel),
 * light colour, strength (clamped to [0,1]).  Before the first call the
 * renderer is unlit (strength 0). */
int pbr_light_set(pbr_ctx* ctx, const float ambient[3], const float direction[3], const float color[3],
                  float strength);

/* Clear colour (renderer/renderer.py:91-94,262); default (0,0,0,1). */
int pbr_background_set(pbr_ctx* ctx, const float rgba[4]);

/* Raster launch configuration.  kernel: 0 = automatic, 1 = scene-per-warp
 * (scenes of at most 64 source triangles, width a multiple of 16),
 * 2 = tile kernel (one CTA per scene region, any scene size).  threads per
 * CTA (128, 256 or 512), bin size of the tile kernel in pixels (8, 16 or 32),
 * its triangle capacity per chunk (0 = automatic) and persistent
 * work-stealing scheduling (0/1).  No counterpart in the reference (the GL
 * driver schedules its own work). */
int pbr_raster_config(pbr_ctx* ctx, int kernel, int threads, int bin_px, int tri_cap, int persistent);

/* The tile kernel's pre-test of small kept triangles: a triangle whose box
 * holds at most 16 pixel centres is kept only if it covers one of them with a
 * depth below the key the chunks drawn so far left there.  The pixels are the
 * same either way; it pays in scenes with many small overlapping triangles.
 * mode -1 (the default): on when a scene holds at least as many source
 * triangles as pixels; 0 off; 1 on.  No reference counterpart. */
int pbr_tile_pretest(pbr_ctx* ctx, int mode);

/* Time the candidate launch configurations on the bound scene and keep the
 * fastest.  d_out is an [N,C,H,W] uint8 scratch image.  Synchronises the
 * stream; do not call during graph capture.  Reports the choice through the
 * out pointers (any may be NULL).  No counterpart in the reference. */
int pbr_autotune(pbr_ctx* ctx, uint8_t* d_out, void* stream, int* out_kernel, int* out_threads,
                 int* out_bin_px, int* out_tri_cap, int* out_persistent, float* out_ms);

/* Render every scene (hard raster): d_out [N,C,H,W] uint8, optional
 * d_depth [N,H,W] float32 window depth (1.0 where nothing is drawn) and
 * optional d_winner [N,H,W] int32 (instance rank within the scene, counted
 * in node order, times the largest mesh's triangle count plus the triangle
 * index; -1 for background).  All three must be 16-byte aligned.
 * Replaces taskMgr.step() + grab_pixels +
 * _rearrange_img (renderer/renderer.py:377-390,326-363). */
int pbr_render(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, int32_t* d_winner, void* stream);

/* pbr_render with the state-bound pose components read from d_state (see
 * pbr_node_bind_state) and written back into the node's pose buffers, as
 * an explicit per-step copy would leave them: one launch for the whole
 * env step.  The source is cleared again before returning.  No reference
 * counterpart (the reference copies state into poses on the host, then
 * draws). */
int pbr_render_state(pbr_ctx* ctx, const float* d_state, long long rows, int cols, long long row_stride,
                     uint8_t* d_out, float* d_depth, int32_t* d_winner, void* stream);

/* "Plain" per-node path that mirrors the reference's per-step flow (one draw
 * per node into a depth/colour buffer, then a readback into [N,C,H,W]):
 * clear, draw one node, resolve.  Uses a context-owned colour+depth buffer
 * allocated on first use (N*H*W*8 bytes). */
int pbr_plain_clear(pbr_ctx* ctx, void* stream);
int pbr_plain_draw(pbr_ctx* ctx, int node_id, void* stream);
int pbr_plain_resolve(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, void* stream);

/* ---- Differentiable soft-coverage mode (no counterpart in the reference) ----
 * Per pixel p and front-facing triangle j: soft coverage
 * D_j = prod_k sigmoid(dist_k(p) / sigma) over the three edge lines (0 beyond
 * 16 sigma outside), normalised linear depth zs_j = (zfar - w)/(zfar - znear),
 * shaded colour C_j (shaders/basic.frag:33-38, unclamped);
 * out = A * softmax_j(zs_j / gamma weighted by D_j) . C + (1 - A) * bg with
 * A = 1 - prod_j (1 - D_j).  Triangles not fully in front of the near plane
 * are dropped.  Defaults: sigma = 0.5 / (2 ln 9) px (0.5 px 10-90 % edge),
 * gamma = 1e-3; threads per CTA 256. */
int pbr_soft_config(pbr_ctx* ctx, float sigma, float gamma, int threads);

/* Gradient buffers of a node (float32, B rows, accumulated with +=; any may be
 * NULL): d_gpos [B,3], d_ghpr [B,3], d_gscale [B], d_gcol [B,4] (alpha gets 0). */
int pbr_node_set_grads(pbr_ctx* ctx, int node_id, float* d_gpos, float* d_ghpr, float* d_gscale, float* d_gcol);

/* Soft forward: d_out [N,3,H,W] float32; d_stats 6*N*H*W float32 (optional,
 * needed by the backward, 16-byte aligned): per pixel the largest normalised
 * depth m, the softmax denominator relative to it, a code for prod(1 - D),
 * and the blended colour relative to the first fragment's colour (dl), stored
 * as N*H*W float4 (m, denominator, code, dl[0]) followed by N*H*W float2
 * (dl[1], dl[2]). */
int pbr_render_soft(pbr_ctx* ctx, float* d_out, float* d_stats, void* stream);

/* Soft adjoint: given the forward's d_out and d_stats and dL/dout
 * d_grad_out [N,3,H,W], accumulate per-instance gradients into the buffers of
 * pbr_node_set_grads and dL/d(normalised light direction) into
 * d_grad_light [3] (optional).  Every node must be in PBR_MODE_HPR.  Fragment
 * lists are recomputed from the triangle setup, nothing per fragment is
 * stored.  Uses float atomics: the summation order is not fixed. */
int pbr_backward_soft(pbr_ctx* ctx, const float* d_out, const float* d_stats, const float* d_grad_out,
                      float* d_grad_light, void* stream);

/* The plain per-node render (clear, one draw per node, resolve) with its
 * depth/colour scratch in a static 16 MiB device array instead of a
 * cudaMalloc'd buffer: for callers that may not allocate device memory when
 * they render -- inside a CUDA stream capture, or under a host framework whose
 * allocator owns the device memory.  The context is created beforehand.
 * Limit: num_scenes * width * height at most about 2M pixels (8 bytes each);
 * larger requests fail with PBR_ERR_CAPACITY.  The first call on a device
 * loads the library's module that holds the array (CUDA loads device code
 * lazily), which reserves its 16 MiB on that device until the process exits,
 * and looks up its device address (cudaGetSymbolAddress): make that first
 * call before any stream capture.  Later calls allocate nothing.  All calls
 * share the one array: calls that overlap on the GPU (other streams, other
 * contexts) race; calls on one stream are ordered.  No counterpart in the
 * reference. */
int pbr_plain_render_noalloc(pbr_ctx* ctx, uint8_t* d_out, float* d_depth, void* stream);

/* Model matrices the kernels build for one node: d_out [B,16] row-major.
 * For tests; replaces reading back matbuf (renderer/node.py:110-126). */
int pbr_debug_transforms(pbr_ctx* ctx, int node_id, float* d_out, void* stream);

/* Device-side error flags accumulated since the last call (synchronises the
 * context's device, then clears them).  0 = none. */
int pbr_device_status(pbr_ctx* ctx, int32_t* out_flags);

/* One CartPole-v0 step for n scenes in a single launch (no context needed):
 * the Euler-integrated dynamics, termination, survival reward and auto-reset
 * of envs/cartpole/env.py:111-218 (_dynamics, _termination, _reward and the
 * auto-reset of _step), evaluated with the same float32 roundings as the
 * reference's tensor operations.
 *   d_obs [n,4] (x, x_dot, theta, theta_dot), d_action [n] int64 (1 = push
 *   right), d_step_count [n] int64 or NULL (all 0);
 *   d_reset_* [n] float32 each: the initial states to use where a scene is done
 *   (required when auto_reset);
 *   outputs: d_next_raw [n,4] (the state after the dynamics: what is drawn),
 *   d_next_obs [n,4] (after auto-reset), d_reward [n], d_done [n] bool bytes,
 *   d_next_step_count [n] int64.  The [n,4] arrays are 16-byte aligned.
 *   consts: gravity, masscart, masspole, length, force_mag, tau, x_threshold,
 *   theta_threshold (radians), max_steps. */
int pbr_cartpole_step(const float* d_obs, const int64_t* d_action, const int64_t* d_step_count,
                      const float* d_reset_x, const float* d_reset_x_dot, const float* d_reset_theta,
                      const float* d_reset_theta_dot, float* d_next_raw, float* d_next_obs, float* d_reward,
                      uint8_t* d_done, int64_t* d_next_step_count, long long n, const double* consts,
                      int auto_reset, void* stream);

/* Per-scene camera matrices in one launch (no context): the view of
 * renderer/camera.py:201-240 and VP = P V of camera.py:252-262, replacing the
 * reference's per-step host math and buffer-texture upload of viewbuf.
 * d_view [K,16] row-major is updated in place: with d_forward and/or d_up
 * given ([K,3]; a missing one keeps the current forward (-row 2) or up (row 1)),
 * f = normalize(forward), up = normalize(up), s = normalize(f x up), u = s x f,
 * rows 0..2 = s, u, -f; with d_eye [K,3] the translation is (-s.e, -u.e, f.e).
 * d_vp [K,16] (or NULL) receives projection (16 floats, row-major, host
 * memory) times the view.  Normalisation divides by max(|v|, 1e-8). */
int pbr_camera_update(const float* d_eye, const float* d_forward, const float* d_up, float* d_view,
                      const float projection[16], float* d_vp, int num_scenes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PBR_CAPI_H */
