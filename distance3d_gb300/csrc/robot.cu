// robot.cu -- forward kinematics of serial chains on the device, for batched
// self-collision checks (the caller of the path in distance3d's
// self_collision.detect, self_collision.py:5-64, with the URDF chain it gets
// from urdf.py, here given directly).
//
// Link 0 is the base (identity).  Joint j (revolute) sits at the fixed
// transform origin_j of link j and turns link j+1 about its unit axis:
//   T_{j+1} = T_j * origin_j * Rot(axis_j, q_j)
// and body b, fixed to link link_b at origin_b, has the pose
//   T_{link_b} * origin_b.
// One thread per (configuration, body) walks the chain up to its link.
// Compiled with -fmad=false; sin/cos are CUDA's.
#include "capi_util.h"

namespace {

// 3x4 transforms: R row-major (9) then t (3), the store's pose layout
__device__ __forceinline__ void compose(const double* A, const double* B, double* C) {
    double R[9], t[3];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j)
            R[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
        t[i] = A[3 * i] * B[9] + A[3 * i + 1] * B[10] + A[3 * i + 2] * B[11] + A[9 + i];
    }
    for (int k = 0; k < 9; ++k) C[k] = R[k];
    for (int k = 0; k < 3; ++k) C[9 + k] = t[k];
}

// rotation by angle q about unit axis a (Rodrigues), no translation
__device__ __forceinline__ void axis_angle(const double* a, double q, double* T) {
    double s, c;
    sincos(q, &s, &c);
    const double C = 1.0 - c;
    const double x = a[0], y = a[1], z = a[2];
    T[0] = c + x * x * C;
    T[1] = x * y * C - z * s;
    T[2] = x * z * C + y * s;
    T[3] = y * x * C + z * s;
    T[4] = c + y * y * C;
    T[5] = y * z * C - x * s;
    T[6] = z * x * C - y * s;
    T[7] = z * y * C + x * s;
    T[8] = c + z * z * C;
    T[9] = T[10] = T[11] = 0.0;
}

__global__ void k_chain_fk(d3d_chain ch, const double* __restrict__ q, int64_t n_configs, double* __restrict__ poses) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_configs * ch.n_bodies) return;
    const int64_t c = k / ch.n_bodies;
    const int b = (int)(k - c * ch.n_bodies);
    const int link = ch.body_link[b];
    double T[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
    for (int j = 0; j < link && j < ch.n_joints; ++j) {
        double O[12], R[12];
        compose(T, ch.joint_origin + 12 * j, O);
        axis_angle(ch.joint_axis + 3 * j, q[c * ch.n_joints + j], R);
        compose(O, R, T);
    }
    compose(T, ch.body_origin + 12 * b, poses + 12 * k);
}

}  // namespace

extern "C" int d3d_chain_fk(const d3d_chain* chain, const double* q, int64_t n_configs, double* poses,
                            void* stream) {
    D3D_REQUIRE(chain && n_configs >= 0, "d3d_chain_fk: invalid argument");
    D3D_REQUIRE(chain->n_joints >= 0 && chain->n_bodies >= 0, "d3d_chain_fk: negative sizes");
    const int64_t n = n_configs * chain->n_bodies;
    if (n == 0) return D3D_SUCCESS;
    D3D_REQUIRE(q && poses && chain->body_link && chain->body_origin &&
                    (chain->n_joints == 0 || (chain->joint_axis && chain->joint_origin)),
                "d3d_chain_fk: null pointer");
    k_chain_fk<<<d3d::grid_for(n, 128), 128, 0, d3d::as_stream(stream)>>>(*chain, q, n_configs, poses);
    return d3d::check_launch("d3d_chain_fk");
}
