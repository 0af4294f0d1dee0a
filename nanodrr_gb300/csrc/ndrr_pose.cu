// Registration pose on the device (ndrr_pose_so3_fwd/bwd): the reference's
// Registration.pose (registration/registration.py:64-68) for the "so3_log"
// parameterisation (geometry/se3.py:179-221),
//   pose = rt_inv @ pivot @ T @ pivot_inv,  T = [[R, R xyz], [0, 1]],
//   R = exp([v]x) = I + a K + b K^2,  K = [v]x,
//   a = sin(t) / t,  b = (1 - cos t) / t^2,  t = |v|,
// and its adjoint to (v, xyz). One thread per pose in float64: the handful
// of 4x4 products replace about thirty elementwise torch launches per
// direction, and float64 keeps b and the derivatives of a and b accurate
// where float32 cancels (t between 1e-4 and 1e-2).
#include <cuda_runtime.h>

#include "../../include/nanodrr_gb300.h"

namespace ndrr {

constexpr int kPoseBlock = 64;

// a, b and their derivatives divided by t (da/dv = ca v, db/dv = cb v).
// Below t = 0.1 the Taylor series (error < 1e-15 there), above it the
// closed forms, whose cancellation in float64 stays below 1e-10 relative.
__device__ __forceinline__ void rodrigues_coefficients(double t2, double& a, double& b, double& ca, double& cb) {
    if (t2 < 1e-2) {
        a = 1.0 + t2 * (-1.0 / 6 + t2 * (1.0 / 120 + t2 * (-1.0 / 5040 + t2 * (1.0 / 362880))));
        b = 0.5 + t2 * (-1.0 / 24 + t2 * (1.0 / 720 + t2 * (-1.0 / 40320 + t2 * (1.0 / 3628800))));
        ca = -1.0 / 3 + t2 * (1.0 / 30 + t2 * (-1.0 / 840 + t2 * (1.0 / 45360)));
        cb = -1.0 / 12 + t2 * (1.0 / 180 + t2 * (-1.0 / 6720 + t2 * (1.0 / 453600)));
    } else {
        const double t = sqrt(t2), s = sin(t), c = cos(t);
        a = s / t;
        b = (1.0 - c) / t2;
        ca = (t * c - s) / (t2 * t);
        cb = (t * s - 2.0 + 2.0 * c) / (t2 * t2);
    }
}

struct PoseTerms {
    double v[3], x[3];
    double K[3][3], K2[3][3], R[3][3];
    double a, b, ca, cb;
};

__device__ __forceinline__ void pose_terms(const float* rot, const float* xyz, int row, PoseTerms& q) {
    for (int i = 0; i < 3; ++i) {
        q.v[i] = (double)rot[row * 3 + i];
        q.x[i] = (double)xyz[row * 3 + i];
    }
    const double vx = q.v[0], vy = q.v[1], vz = q.v[2];
    const double K[3][3] = {{0.0, -vz, vy}, {vz, 0.0, -vx}, {-vy, vx, 0.0}};
    rodrigues_coefficients(vx * vx + vy * vy + vz * vz, q.a, q.b, q.ca, q.cb);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            q.K[i][j] = K[i][j];
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += K[i][k] * K[k][j];
            q.K2[i][j] = s;
            q.R[i][j] = (i == j ? 1.0 : 0.0) + q.a * K[i][j] + q.b * s;
        }
}

__device__ __forceinline__ void load44(const float* m, double (&o)[4][4]) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) o[i][j] = (double)m[i * 4 + j];
}

__device__ __forceinline__ void mul44(const double (&A)[4][4], const double (&B)[4][4], double (&C)[4][4]) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += A[i][k] * B[k][j];
            C[i][j] = s;
        }
}

__global__ void __launch_bounds__(kPoseBlock) pose_so3_fwd_kernel(const float* __restrict__ rot,
                                                                  const float* __restrict__ xyz, int param_rows,
                                                                  const float* __restrict__ rt_inv,
                                                                  const float* __restrict__ pivot,
                                                                  const float* __restrict__ pivot_inv, int B,
                                                                  float* __restrict__ pose) {
    const int b = blockIdx.x * kPoseBlock + threadIdx.x;
    if (b >= B) return;
    PoseTerms q;
    pose_terms(rot, xyz, param_rows == 1 ? 0 : b, q);
    double T[4][4], A[4][4], P[4][4], C[4][4], AT[4][4], out[4][4];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) T[i][j] = q.R[i][j];
        T[i][3] = q.R[i][0] * q.x[0] + q.R[i][1] * q.x[1] + q.R[i][2] * q.x[2];
    }
    T[3][0] = T[3][1] = T[3][2] = 0.0;
    T[3][3] = 1.0;
    load44(rt_inv + (size_t)b * 16, A);
    load44(pivot + (size_t)b * 16, P);
    load44(pivot_inv + (size_t)b * 16, C);
    double AP[4][4];
    mul44(A, P, AP);
    mul44(AP, T, AT);
    mul44(AT, C, out);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) pose[(size_t)b * 16 + i * 4 + j] = (float)out[i][j];
}

// gT = (rt_inv pivot)^T gpose pivot_inv^T; gR = gT[:3, :3] + gT[:3, 3] xyz^T,
// g_xyz = R^T gT[:3, 3]; g_v = (ca <gR, K> + cb <gR, K^2>) v + a vee(gR)
// + b vee(gR K^T + K^T gR), with vee(G) = (G21 - G12, G02 - G20, G10 - G01)
// the gradient of <G, [v]x> in v.
__global__ void __launch_bounds__(kPoseBlock) pose_so3_bwd_kernel(const float* __restrict__ gpose,
                                                                  const float* __restrict__ rot,
                                                                  const float* __restrict__ xyz, int param_rows,
                                                                  const float* __restrict__ rt_inv,
                                                                  const float* __restrict__ pivot,
                                                                  const float* __restrict__ pivot_inv, int B,
                                                                  float* __restrict__ g_rot,
                                                                  float* __restrict__ g_xyz) {
    const int b = blockIdx.x * kPoseBlock + threadIdx.x;
    if (b >= B) return;
    PoseTerms q;
    pose_terms(rot, xyz, param_rows == 1 ? 0 : b, q);
    double A[4][4], P[4][4], C[4][4], G[4][4], AP[4][4], L[4][4], gT[4][4];
    load44(rt_inv + (size_t)b * 16, A);
    load44(pivot + (size_t)b * 16, P);
    load44(pivot_inv + (size_t)b * 16, C);
    load44(gpose + (size_t)b * 16, G);
    mul44(A, P, AP);
    // L = AP^T G, gT = L C^T
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += AP[k][i] * G[k][j];
            L[i][j] = s;
        }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += L[i][k] * C[j][k];
            gT[i][j] = s;
        }
    double gR[3][3], sK = 0.0, sK2 = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            gR[i][j] = gT[i][j] + gT[i][3] * q.x[j];
            sK += gR[i][j] * q.K[i][j];
            sK2 += gR[i][j] * q.K2[i][j];
        }
    for (int j = 0; j < 3; ++j)
        g_xyz[(size_t)b * 3 + j] = (float)(q.R[0][j] * gT[0][3] + q.R[1][j] * gT[1][3] + q.R[2][j] * gT[2][3]);
    // H = gR K^T + K^T gR
    double H[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += gR[i][k] * q.K[j][k] + q.K[k][i] * gR[k][j];
            H[i][j] = s;
        }
    const double radial = q.ca * sK + q.cb * sK2;
    const double vr[3] = {gR[2][1] - gR[1][2], gR[0][2] - gR[2][0], gR[1][0] - gR[0][1]};
    const double vh[3] = {H[2][1] - H[1][2], H[0][2] - H[2][0], H[1][0] - H[0][1]};
    for (int i = 0; i < 3; ++i) g_rot[(size_t)b * 3 + i] = (float)(radial * q.v[i] + q.a * vr[i] + q.b * vh[i]);
}

cudaError_t launch_pose_fwd(const float* rot, const float* xyz, int param_rows, const float* rt_inv,
                            const float* pivot, const float* pivot_inv, int B, float* pose, cudaStream_t st) {
    pose_so3_fwd_kernel<<<(B + kPoseBlock - 1) / kPoseBlock, kPoseBlock, 0, st>>>(rot, xyz, param_rows, rt_inv,
                                                                                  pivot, pivot_inv, B, pose);
    return cudaGetLastError();
}

cudaError_t launch_pose_bwd(const float* gpose, const float* rot, const float* xyz, int param_rows,
                            const float* rt_inv, const float* pivot, const float* pivot_inv, int B, float* g_rot,
                            float* g_xyz, cudaStream_t st) {
    pose_so3_bwd_kernel<<<(B + kPoseBlock - 1) / kPoseBlock, kPoseBlock, 0, st>>>(
        gpose, rot, xyz, param_rows, rt_inv, pivot, pivot_inv, B, g_rot, g_xyz);
    return cudaGetLastError();
}

}  // namespace ndrr
