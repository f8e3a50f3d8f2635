// 3x3 rotation-variant SVD for the ARAP constraint, single precision.
//
// F = U diag(s) V^T with U, V proper rotations; s is sorted by decreasing
// magnitude and the sign of det F sits on s[2] (the convention of the
// reference's ti.svd, cons/mgpbd_gpu.py:236).  Method:
//  1. eigen-decomposition of the symmetric M = F^T F - I by cyclic Jacobi
//     rotations (Golub & Van Loan, "Matrix Computations", 4th ed., sec.
//     8.5.2-8.5.3; rotation from the Rutishauser formulas t = sgn(tau) /
//     (|tau| + sqrt(1 + tau^2))).  Forming M from G = F - I as G + G^T + G^T G
//     keeps the small deviations of near-rigid tets instead of rounding them
//     against the identity.
//  2. columns of V sorted by decreasing eigenvalue, det V forced to +1;
//  3. B = F V, Gram-Schmidt QR with u3 = u1 x u2 so det U = +1: s1 = |b1|,
//     s2 = u2.b2 >= 0, s3 = u3.b3 carries the sign of det F.  Degenerate
//     columns fall back to an arbitrary orthonormal completion.
#pragma once

#include <cuda_runtime.h>

namespace mgpbd {

struct Mat3 {
  float m[3][3];  // m[row][col]
};

__host__ __device__ inline void jacobi_rotate(float (&a)[3][3], float (&v)[3][3], int p, int q) {
  float apq = a[p][q];
  if (apq == 0.0f) return;
  float app = a[p][p], aqq = a[q][q];
  float tau = (aqq - app) / (2.0f * apq);
  float t = (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
  float c = 1.0f / sqrtf(1.0f + t * t);
  float s = t * c;
  // A' = J^T A J with J the (p,q) rotation [c s; -s c]
  for (int k = 0; k < 3; ++k) {
    float akp = a[k][p], akq = a[k][q];
    a[k][p] = c * akp - s * akq;
    a[k][q] = s * akp + c * akq;
  }
  for (int k = 0; k < 3; ++k) {
    float apk = a[p][k], aqk = a[q][k];
    a[p][k] = c * apk - s * aqk;
    a[q][k] = s * apk + c * aqk;
  }
  a[p][q] = a[q][p] = 0.0f;
  for (int k = 0; k < 3; ++k) {
    float vkp = v[k][p], vkq = v[k][q];
    v[k][p] = c * vkp - s * vkq;
    v[k][q] = s * vkp + c * vkq;
  }
}

__host__ __device__ inline void normalize3(float (&x)[3], float& len) {
  len = sqrtf(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  float inv = len > 0.0f ? 1.0f / len : 0.0f;
  x[0] *= inv;
  x[1] *= inv;
  x[2] *= inv;
}

// Unit vector orthogonal to unit u (for degenerate columns).
__host__ __device__ inline void any_orthogonal(const float (&u)[3], float (&o)[3]) {
  // cross with the axis least aligned with u
  float ax = fabsf(u[0]), ay = fabsf(u[1]), az = fabsf(u[2]);
  float e[3] = {0.0f, 0.0f, 0.0f};
  if (ax <= ay && ax <= az) e[0] = 1.0f;
  else if (ay <= az) e[1] = 1.0f;
  else e[2] = 1.0f;
  o[0] = u[1] * e[2] - u[2] * e[1];
  o[1] = u[2] * e[0] - u[0] * e[2];
  o[2] = u[0] * e[1] - u[1] * e[0];
  float l;
  normalize3(o, l);
}

__host__ __device__ inline void svd3_rv(const float (&F)[3][3], float (&U)[3][3], float (&s)[3],
                                        float (&V)[3][3]) {
  // M = G + G^T + G^T G, G = F - I
  float G[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) G[i][j] = F[i][j] - (i == j ? 1.0f : 0.0f);
  float a[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      float gtg = G[0][i] * G[0][j] + G[1][i] * G[1][j] + G[2][i] * G[2][j];
      a[i][j] = G[i][j] + G[j][i] + gtg;
      a[j][i] = a[i][j];
    }
  float v[3][3] = {{1.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}};
#pragma unroll 1
  for (int sweep = 0; sweep < 6; ++sweep) {
    float off = fabsf(a[0][1]) + fabsf(a[0][2]) + fabsf(a[1][2]);
    float dia = fabsf(a[0][0]) + fabsf(a[1][1]) + fabsf(a[2][2]);
    if (off <= 1e-12f * dia || off == 0.0f) break;
    jacobi_rotate(a, v, 0, 1);
    jacobi_rotate(a, v, 0, 2);
    jacobi_rotate(a, v, 1, 2);
  }
  // sort eigenvalues (of M; sigma^2 = 1 + mu) in decreasing order
  float mu[3] = {a[0][0], a[1][1], a[2][2]};
  int idx[3] = {0, 1, 2};
  if (mu[idx[0]] < mu[idx[1]]) { int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
  if (mu[idx[1]] < mu[idx[2]]) { int t = idx[1]; idx[1] = idx[2]; idx[2] = t; }
  if (mu[idx[0]] < mu[idx[1]]) { int t = idx[0]; idx[0] = idx[1]; idx[1] = t; }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = v[i][idx[j]];
  float detv = V[0][0] * (V[1][1] * V[2][2] - V[1][2] * V[2][1]) -
               V[0][1] * (V[1][0] * V[2][2] - V[1][2] * V[2][0]) +
               V[0][2] * (V[1][0] * V[2][1] - V[1][1] * V[2][0]);
  if (detv < 0.0f) {
    V[0][2] = -V[0][2];
    V[1][2] = -V[1][2];
    V[2][2] = -V[2][2];
  }
  // B = F V
  float b[3][3];  // b[col][row]
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) b[c][r] = F[r][0] * V[0][c] + F[r][1] * V[1][c] + F[r][2] * V[2][c];
  float u1[3] = {b[0][0], b[0][1], b[0][2]};
  float l1;
  normalize3(u1, l1);
  if (!(l1 > 1e-30f)) {
    u1[0] = 1.0f;
    u1[1] = 0.0f;
    u1[2] = 0.0f;
    l1 = 0.0f;
  }
  float d12 = u1[0] * b[1][0] + u1[1] * b[1][1] + u1[2] * b[1][2];
  float u2[3] = {b[1][0] - d12 * u1[0], b[1][1] - d12 * u1[1], b[1][2] - d12 * u1[2]};
  float l2;
  normalize3(u2, l2);
  if (!(l2 > 1e-30f)) {
    any_orthogonal(u1, u2);
    l2 = 0.0f;
  }
  float u3[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2],
                 u1[0] * u2[1] - u1[1] * u2[0]};
  s[0] = l1;
  s[1] = u2[0] * b[1][0] + u2[1] * b[1][1] + u2[2] * b[1][2];
  s[2] = u3[0] * b[2][0] + u3[1] * b[2][1] + u3[2] * b[2][2];
  for (int r = 0; r < 3; ++r) {
    U[r][0] = u1[r];
    U[r][1] = u2[r];
    U[r][2] = u3[r];
  }
}

}  // namespace mgpbd
