// lumrad_blockify.cpp — the producers of a frame's world and palette for animated voxel models:
// blockify (host) and map (device).
//
// In the reference, each frame (Renderer::submitFrame, renderer.cpp:428-455):
//   start_blockify   current_world = origin_world; temporary slots start at static_block_palette_size
//                    (internal_render.cpp:977-986)
//   blockify_mesh    every block under a mesh's AABB whose id is static gets a fresh temporary slot,
//                    queued to receive a copy of the static block's voxels (:1031-1070)
//   exec_copies      the palette's temporary part is cleared, the queued copies run, the world is
//                    uploaded (:1375-1476)
//   map_mesh         map.comp writes each mesh's voxels into the temporary blocks through the
//                    inverse transform (:1484-1520, shaders/map.comp)
// lumrad_blockify does all four for a list of meshes; the passes after it read the blockified
// world and palette (one call = one frame's producers), the origin world stays as loaded.
//
// Transform math follows glm as the reference calls it: toMat4(quat) in float, translate on the
// identity, shift * rotate = [R | s] exactly; the AABB of the model's corners through
// dmat4 * vec4 (pairwise sums (m0*v0 + m1*v1) + (m2*v2 + m3*v3) in double, rounded to float).
// The inverse of [R | s] is the rigid inverse [R^T | -R^T s] in double rounded to float (glm's
// general inverse agrees up to the double rounding).  Where several map invocations target one
// palette voxel (the reference races), the result is as if the invocations ran one after another
// in linear order (x fastest) and the meshes in order.

#include "lumrad_world.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace lumrad {
namespace {

// glm::mat3_cast of quaternion (x, y, z, w), float arithmetic; r[col][row]
void quat_to_mat(const float q[4], float r[3][3]) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    const float xx = x * x, yy = y * y, zz = z * z, xz = x * z, xy = x * y, yz = y * z;
    const float wx = w * x, wy = w * y, wz = w * z;
    r[0][0] = 1.0f - 2.0f * (yy + zz);
    r[0][1] = 2.0f * (xy + wz);
    r[0][2] = 2.0f * (xz - wy);
    r[1][0] = 2.0f * (xy - wz);
    r[1][1] = 1.0f - 2.0f * (xx + zz);
    r[1][2] = 2.0f * (yz + wx);
    r[2][0] = 2.0f * (xz + wy);
    r[2][1] = 2.0f * (yz - wx);
    r[2][2] = 1.0f - 2.0f * (xx + yy);
}

struct Box { float mn[3], mx[3]; };

// get_shift (internal_render.cpp:988-1012): AABB of the 8 corners of (size - 1) through [R | s]
Box model_aabb(const float r[3][3], const float s[3], const int size[3]) {
    const float b[3] = {(float)(size[0] - 1), (float)(size[1] - 1), (float)(size[2] - 1)};
    const float corners[8][3] = {{0, 0, 0}, {0, b[1], 0}, {0, b[1], b[2]}, {0, 0, b[2]},
                                 {b[0], 0, 0}, {b[0], b[1], 0}, {b[0], b[1], b[2]}, {b[0], 0, b[2]}};
    Box box;
    for (int a = 0; a < 3; a++) {
        box.mn[a] = 3.40282347e38f;
        box.mx[a] = -3.40282347e38f;
    }
    for (const auto& c : corners)
        for (int a = 0; a < 3; a++) {
            const double p = ((double)r[0][a] * c[0] + (double)r[1][a] * c[1]) +
                             ((double)r[2][a] * c[2] + (double)s[a] * 1.0);
            const float pf = (float)p;
            box.mn[a] = pf < box.mn[a] ? pf : box.mn[a];
            box.mx[a] = box.mx[a] < pf ? pf : box.mx[a];
        }
    return box;
}

int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace
}  // namespace lumrad

using namespace lumrad;

extern "C" {

int lumrad_load_model(LumRadContext ctx, const uint8_t* voxels, int sx, int sy, int sz, int* model) {
    Context* c = as_ctx(ctx);
    if (!c || !voxels || !model) return fail(LUMRAD_EINVAL, "null argument");
    if (sx < 1 || sy < 1 || sz < 1 || sx > 1024 || sy > 1024 || sz > 1024)
        return fail(LUMRAD_EINVAL, "model size must be in [1, 1024] per axis");
    LUMRAD_TRY(cudaSetDevice(c->device));
    Context::Model m;
    m.sx = sx; m.sy = sy; m.sz = sz;
    const size_t bytes = (size_t)sx * sy * sz;
    LUMRAD_TRY(cudaMalloc(&m.d_vox, bytes));
    const cudaError_t e = cudaMemcpy(m.d_vox, voxels, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(m.d_vox);
        return fail(LUMRAD_EDEVICE, std::string("model upload: ") + cudaGetErrorString(e));
    }
    c->models.push_back(m);
    *model = (int)c->models.size() - 1;
    return LUMRAD_OK;
}

int lumrad_blockify(LumRadContext ctx, int static_blocks, const int* models, const LumRadMeshTransform* transforms,
                    int n_meshes) {
    Context* c = as_ctx(ctx);
    if (!c || n_meshes < 0 || (n_meshes > 0 && (!models || !transforms))) return fail(LUMRAD_EINVAL, "bad argument");
    if (int rc = check_unowned(c)) return rc;
    NvtxRange range("lumrad blockify");
    DeviceWorld& w = c->world;
    if (static_blocks < 1 || static_blocks > w.n_slots) return fail(LUMRAD_EINVAL, "static_blocks must be in [1, max_block_types]");
    if (n_meshes >= (1 << 23)) return fail(LUMRAD_EINVAL, "too many meshes");
    for (int i = 0; i < n_meshes; i++)
        if (models[i] < 0 || models[i] >= (int)c->models.size()) return fail(LUMRAD_EINVAL, "unknown model");
    LUMRAD_TRY(cudaSetDevice(c->device));
    int rc = w.sync_inputs(c->stream);   // the origin world and palette as loaded
    if (rc) return rc;

    // page-locked staging (see Context::h_blk), made on the first call
    const size_t off_cgrid = w.W * sizeof(int16_t), off_cslot = off_cgrid + w.W * sizeof(uint16_t);
    const size_t n_cslot = (size_t)w.n_slots + 128;
    const size_t off_copies = off_cslot + n_cslot * sizeof(int);
    if (!c->h_blk) {
        LUMRAD_TRY(cudaMallocHost(&c->h_blk, off_copies + (size_t)w.n_slots * sizeof(int2)));
        LUMRAD_TRY(cudaMalloc(&c->d_blk_copies, (size_t)w.n_slots * sizeof(int2)));
    }
    int16_t* cur = reinterpret_cast<int16_t*>(c->h_blk);   // the previous call's uploads are done
    int2* copies = reinterpret_cast<int2*>(c->h_blk + off_copies);
    std::memcpy(cur, w.h_grid.data(), w.W * sizeof(int16_t));
    int n_copies = 0;

    // blockify (host): temporary slots from static_blocks up, in mesh order
    int counter = static_blocks;
    for (int i = 0; i < n_meshes; i++) {
        float r[3][3];
        quat_to_mat(transforms[i].rot, r);
        const Context::Model& m = c->models[models[i]];
        const int size[3] = {m.sx, m.sy, m.sz};
        const Box box = model_aabb(r, transforms[i].shift, size);
        const int ws[3] = {w.X, w.Y, w.Z};
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {   // (ivec3(min) - 1) / 16, (ivec3(max) + 1) / 16, clamped (:1037-1041)
            lo[a] = clampi(((int)box.mn[a] - 1) / 16, 0, ws[a] - 1);
            hi[a] = clampi(((int)box.mx[a] + 1) / 16, 0, ws[a] - 1);
        }
        for (int z = lo[2]; z <= hi[2]; z++)
            for (int y = lo[1]; y <= hi[1]; y++)
                for (int x = lo[0]; x <= hi[0]; x++) {
                    int16_t& b = cur[(size_t)x + (size_t)w.X * ((size_t)y + (size_t)w.Y * z)];
                    if (b >= static_blocks) continue;   // already temporary (or a dynamic id): left as is
                    if (counter >= w.n_slots || counter > 32767)
                        return fail(LUMRAD_ENOMEM, "temporary blocks exceed max_block_types");
                    // copy the static block's voxels; a negative id has no source block (the
                    // reference's copy would start at a negative palette offset)
                    if (b > 0) copies[n_copies++] = make_int2(b, counter);
                    b = (int16_t)counter++;
                }
    }

    // map dispatches of every mesh (checked before anything reaches the device)
    std::vector<MapArgs> margs(n_meshes);
    for (int i = 0; i < n_meshes; i++) {
        float r[3][3];
        quat_to_mat(transforms[i].rot, r);
        const float* s = transforms[i].shift;
        const Context::Model& m = c->models[models[i]];
        const int size[3] = {m.sx, m.sy, m.sz};
        const Box box = model_aabb(r, s, size);
        MapArgs& a = margs[i];
        double invocations = 1.0;
        for (int k = 0; k < 3; k++) {
            const int mn = (int)std::floor(box.mn[k]);   // ivec3(floor(min)), ivec3(ceil(max)) (:1500-1501)
            const int mx = (int)std::ceil(box.mx[k]);
            a.shift[k] = mn;
            a.dims[k] = (mx - mn + 3) / 4 * 4;   // (map_area + 3) / 4 groups of 4 (:1512)
            invocations *= (double)a.dims[k];
        }
        if (invocations >= 4294967296.0) return fail(LUMRAD_EINVAL, "a mesh covers more than 2^32 world voxels");
        // inverse [R^T | -R^T s], column-major
        for (int col = 0; col < 3; col++)
            for (int row = 0; row < 3; row++) a.inv[4 * col + row] = r[row][col];
        for (int row = 0; row < 3; row++) {
            const double t = ((double)r[row][0] * s[0] + (double)r[row][1] * s[1]) + (double)r[row][2] * s[2];
            a.inv[12 + row] = (float)(-t);
            a.inv[4 * row + 3] = 0.0f;
        }
        a.inv[15] = 1.0f;
    }

    // the slots this frame writes: every id from static_blocks up present in the grid (made here
    // or set by the caller), below n_slots
    int used_end = static_blocks;
    for (size_t i = 0; i < w.W; i++) used_end = std::max(used_end, (int)cur[i] + 1);
    used_end = std::min(used_end, w.n_slots);
    // exec_copies (device): temporary part of the palette cleared (the slots that may hold voxels:
    // the rest are zero already), block copies, world upload
    const int clear_end = std::min(std::max(used_end, w.pal_dirty_end), w.n_slots);
    if (clear_end > static_blocks)
        LUMRAD_TRY(cudaMemsetAsync(w.d_pal + (size_t)static_blocks * 4096, 0, (size_t)(clear_end - static_blocks) * 4096,
                                   c->stream));
    w.pal_dirty_end = used_end;
    if (n_copies > 0) {
        LUMRAD_TRY(cudaMemcpyAsync(c->d_blk_copies, copies, (size_t)n_copies * sizeof(int2), cudaMemcpyHostToDevice,
                                   c->stream));
        LUMRAD_TRY(launch_palette_copies(w.d_pal, c->d_blk_copies, n_copies, c->stream));
    }
    LUMRAD_TRY(cudaMemcpyAsync(w.d_grid, cur, w.W * sizeof(int16_t), cudaMemcpyHostToDevice, c->stream));

    // map (device), mesh by mesh; writes claimed in the owner words (one per voxel of the slots
    // in use: the map writes only into blocks of the grid), then resolved
    const size_t n_tmp = (size_t)(used_end - static_blocks) * 4096;
    if (n_meshes > 0 && n_tmp > 0) {
        if (n_tmp > c->map_owner_cap) {
            LUMRAD_TRY(cudaStreamSynchronize(c->stream));
            cudaFree(c->d_map_owner);
            c->d_map_owner = nullptr;
            c->map_owner_cap = 0;
            LUMRAD_TRY(cudaMalloc(&c->d_map_owner, n_tmp * sizeof(unsigned long long)));
            c->map_owner_cap = n_tmp;
        }
        LUMRAD_TRY(cudaMemsetAsync(c->d_map_owner, 0, n_tmp * sizeof(unsigned long long), c->stream));
    }
    for (int i = 0; i < n_meshes && n_tmp > 0; i++) {
        const Context::Model& m = c->models[models[i]];
        LUMRAD_TRY(launch_map(w.d_grid, w.X, w.Y, w.Z, w.n_slots, static_blocks, m.d_vox, m.sx, m.sy, m.sz, margs[i], i,
                              c->d_map_owner, c->stream));
    }
    if (n_meshes > 0 && n_tmp > 0)
        LUMRAD_TRY(launch_map_resolve(w.d_pal + (size_t)static_blocks * 4096, c->d_map_owner, n_tmp, c->stream));

    // compact world of the blockified grid; occupancy masks from the device palette
    w.build_compact(cur, false);   // the occupancy masks come from the device palette below
    const size_t cap = std::max<size_t>((size_t)w.n_compact, (size_t)w.n_slots + 64);
    if (cap > w.cbits_cap) {
        LUMRAD_TRY(cudaStreamSynchronize(c->stream));
        cudaFree(w.d_cbits);
        cudaFree(w.d_cslot);
        w.d_cbits = nullptr;
        w.d_cslot = nullptr;
        w.cbits_cap = 0;
        LUMRAD_TRY(cudaMalloc(&w.d_cbits, cap * 128 * sizeof(uint32_t)));
        LUMRAD_TRY(cudaMalloc(&w.d_cslot, cap * sizeof(int)));
        w.cbits_cap = cap;
    }
    // the compact grid and slots through the staging area (both fit: at most W uint16 ids, and
    // at most n_slots + 66 compact ids)
    const void* cslot_src = w.h_cslot.data();
    if (w.h_cslot.size() <= n_cslot) {
        std::memcpy(c->h_blk + off_cslot, w.h_cslot.data(), w.h_cslot.size() * sizeof(int));
        cslot_src = c->h_blk + off_cslot;
    }
    std::memcpy(c->h_blk + off_cgrid, w.h_cgrid.data(), w.h_cgrid.size());
    LUMRAD_TRY(cudaMemcpyAsync(w.d_cslot, cslot_src, w.h_cslot.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    LUMRAD_TRY(launch_compact_bits(w.d_pal, w.d_cslot, w.n_compact, w.d_cbits, c->stream));
    LUMRAD_TRY(cudaMemcpyAsync(w.d_cgrid, c->h_blk + off_cgrid, w.h_cgrid.size(), cudaMemcpyHostToDevice, c->stream));
    w.h_cur.assign(cur, cur + w.W);
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));   // the staging area is reused by the next call
    return LUMRAD_OK;
}

int lumrad_get_world(LumRadContext ctx, int16_t* blocks) {
    Context* c = as_ctx(ctx);
    if (!c || !blocks) return fail(LUMRAD_EINVAL, "null argument");
    const DeviceWorld& w = c->world;
    const std::vector<int16_t>& g = w.h_cur.empty() ? w.h_grid : w.h_cur;
    std::memcpy(blocks, g.data(), w.W * sizeof(int16_t));
    return LUMRAD_OK;
}

int lumrad_get_block_palette(LumRadContext ctx, uint8_t* voxels) {
    Context* c = as_ctx(ctx);
    if (!c || !voxels) return fail(LUMRAD_EINVAL, "null argument");
    LUMRAD_TRY(cudaSetDevice(c->device));
    const DeviceWorld& w = c->world;
    LUMRAD_TRY(cudaMemcpyAsync(voxels, w.d_pal, (size_t)w.n_slots * 4096, cudaMemcpyDeviceToHost, c->stream));
    LUMRAD_TRY(cudaStreamSynchronize(c->stream));
    return LUMRAD_OK;
}

}  // extern "C"
