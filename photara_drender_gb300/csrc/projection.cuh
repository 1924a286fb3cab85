// The tests shaders/project_texture.hlsl applies to a texel before it reads the view's visibility:
// in front of the camera, inside the clip volume, inside the viewport and facing the camera at
// least min_view_cosine. Shared by the projection kernel and the ray caster, which traces only the
// texel-views that pass, so both decide identically.
#pragma once

#include <cuda_runtime.h>

#include "../../include/pdr_capi.h"

namespace pdr {

struct ProjectedTexel {
    float ppx, ppy, ndz;  // pixel position and NDC depth
    float vl, cosv;       // distance to the camera and cosine of the view angle
};

__device__ __forceinline__ bool project_texel(const pdr_projection_view& v, float px, float py, float pz, float nx,
                                              float ny, float nz, ProjectedTexel& o) {
    const float* M = v.world_to_clip;
    const float cw = M[12] * px + M[13] * py + M[14] * pz + M[15] * 1.0f;
    if (cw <= 1e-8f) return false;
    const float cx = M[0] * px + M[1] * py + M[2] * pz + M[3] * 1.0f;
    const float cy = M[4] * px + M[5] * py + M[6] * pz + M[7] * 1.0f;
    const float cz = M[8] * px + M[9] * py + M[10] * pz + M[11] * 1.0f;
    const float ndx = cx / cw, ndy = cy / cw, ndz = cz / cw;
    if (ndx < -1.0f || ndy < -1.0f || ndx > 1.0f || ndy > 1.0f || ndz < -1.0f || ndz > 1.0f) return false;
    const float ppx = v.viewport[0] + (ndx * 0.5f + 0.5f) * v.viewport[2];
    const float ppy = v.viewport[1] + (ndy * 0.5f + 0.5f) * v.viewport[3];
    if (ppx < v.viewport[0] || ppy < v.viewport[1] || ppx >= v.viewport[0] + v.viewport[2] ||
        ppy >= v.viewport[1] + v.viewport[3])
        return false;
    // view direction before visibility: the facing test rejects half of all texel-views before the
    // visibility work, with the same outcome as the reference's order
    const float vx0 = v.camera_position[0] - px, vy0 = v.camera_position[1] - py;
    const float vz0 = v.camera_position[2] - pz;
    const float vl = sqrtf(vx0 * vx0 + vy0 * vy0 + vz0 * vz0);
    const float cosv = nx * (vx0 / vl) + ny * (vy0 / vl) + nz * (vz0 / vl);
    if (cosv < v.min_view_cosine) return false;
    o.ppx = ppx;
    o.ppy = ppy;
    o.ndz = ndz;
    o.vl = vl;
    o.cosv = cosv;
    return true;
}

}  // namespace pdr
