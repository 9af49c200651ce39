// Vertex deformation on the GPU: the per-frame vertex work of the
// reference's Renderer::updateScene (src/renderer.cpp:1155-1230), which it
// does on the host and uploads. Here only the pose (a few matrices per mesh
// node and joint) travels; one thread per vertex computes
//   position = (world * skin) * (p, 1),  skin = sum_k weight_k * joint_k
//   normal   = normalMatrix(world) * n
// with every multiply and add rounded separately in the host restatement's
// order (glm's matrix products), so the result matches the host
// evaluation bit for bit. The emissive-triangle vertices follow.
#include "engine.h"

namespace {

__global__ void __launch_bounds__(256) kDeform(uint32_t nv, const float *__restrict__ restP,
                                               const float *__restrict__ restN, const uint32_t *__restrict__ vShape,
                                               const ushort4 *__restrict__ joints, const float4 *__restrict__ weights,
                                               const float *__restrict__ shapeM, const float *__restrict__ shapeN,
                                               const float *__restrict__ jointM, uint32_t numShapes,
                                               uint32_t numJoints, float *__restrict__ outP,
                                               float *__restrict__ outN)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    const uint32_t shape = __ldg(vShape + v);
    if (shape >= numShapes)
        return;
    const float *G = shapeM + 16 * (size_t)shape;
    float P[16];
    const float4 wt = weights ? __ldg(weights + v) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool skinned = joints && (wt.x != 0.0f || wt.y != 0.0f || wt.z != 0.0f || wt.w != 0.0f);
    if (skinned) {
        const ushort4 j = __ldg(joints + v);
        if (j.x >= numJoints || j.y >= numJoints || j.z >= numJoints || j.w >= numJoints)
            return;
        const float *J0 = jointM + 16 * (size_t)j.x, *J1 = jointM + 16 * (size_t)j.y, *J2 = jointM + 16 * (size_t)j.z,
                    *J3 = jointM + 16 * (size_t)j.w;
        float S[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) {
            float acc = __fmul_rn(wt.x, __ldg(J0 + e));
            acc = __fadd_rn(acc, __fmul_rn(wt.y, __ldg(J1 + e)));
            acc = __fadd_rn(acc, __fmul_rn(wt.z, __ldg(J2 + e)));
            acc = __fadd_rn(acc, __fmul_rn(wt.w, __ldg(J3 + e)));
            S[e] = acc;
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float acc = __fmul_rn(__ldg(G + r), S[c * 4]);
                acc = __fadd_rn(acc, __fmul_rn(__ldg(G + 4 + r), S[c * 4 + 1]));
                acc = __fadd_rn(acc, __fmul_rn(__ldg(G + 8 + r), S[c * 4 + 2]));
                acc = __fadd_rn(acc, __fmul_rn(__ldg(G + 12 + r), S[c * 4 + 3]));
                P[c * 4 + r] = acc;
            }
    } else {
#pragma unroll
        for (int e = 0; e < 16; ++e)
            P[e] = __ldg(G + e);
    }
    const float px = __ldg(restP + 3 * (size_t)v), py = __ldg(restP + 3 * (size_t)v + 1),
                pz = __ldg(restP + 3 * (size_t)v + 2);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float acc = __fmul_rn(P[r], px);
        acc = __fadd_rn(acc, __fmul_rn(P[4 + r], py));
        acc = __fadd_rn(acc, __fmul_rn(P[8 + r], pz));
        acc = __fadd_rn(acc, P[12 + r]);
        outP[3 * (size_t)v + r] = acc;
    }
    if (restN && outN) {
        const float *N = shapeN + 9 * (size_t)shape;
        const float nx = __ldg(restN + 3 * (size_t)v), ny = __ldg(restN + 3 * (size_t)v + 1),
                    nz = __ldg(restN + 3 * (size_t)v + 2);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            float acc = __fmul_rn(__ldg(N + 3 * r), nx);
            acc = __fadd_rn(acc, __fmul_rn(__ldg(N + 3 * r + 1), ny));
            acc = __fadd_rn(acc, __fmul_rn(__ldg(N + 3 * r + 2), nz));
            outN[3 * (size_t)v + r] = acc;
        }
    }
}

// Emissive-triangle vertices (float4 x 3 per emitter) from the positions.
__global__ void kEmissiveVerts(int numEmis, const int *__restrict__ emisPrim, const float *__restrict__ pos,
                               const int *__restrict__ idx, int numTris, float4 *__restrict__ emisV)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= numEmis)
        return;
    const int p = __ldg(emisPrim + e);
    if (p < 0 || p >= numTris)
        return;
    for (int k = 0; k < 3; ++k) {
        const int vi = __ldg(idx + 3 * p + k);
        emisV[3 * e + k] = make_float4(__ldg(pos + 3 * (size_t)vi), __ldg(pos + 3 * (size_t)vi + 1),
                                       __ldg(pos + 3 * (size_t)vi + 2), 0.0f);
    }
}

}  // namespace

void launchDeform(uint32_t nv, const float *restP, const float *restN, const uint32_t *vShape, const void *joints,
                  const void *weights, const float *shapeM, const float *shapeN, const float *jointM,
                  uint32_t numShapes, uint32_t numJoints, float *outP, float *outN, cudaStream_t st)
{
    if (nv == 0)
        return;
    kDeform<<<(nv + 255) / 256, 256, 0, st>>>(nv, restP, restN, vShape, static_cast<const ushort4 *>(joints),
                                              static_cast<const float4 *>(weights), shapeM, shapeN, jointM,
                                              numShapes, numJoints, outP, outN);
}

void launchEmissiveVerts(int numEmis, const int *emisPrim, const float *pos, const int *idx, int numTris,
                         float4 *emisV, cudaStream_t st)
{
    if (numEmis <= 0)
        return;
    kEmissiveVerts<<<(numEmis + 127) / 128, 128, 0, st>>>(numEmis, emisPrim, pos, idx, numTris, emisV);
}
