// CPU port of the MGPBD step (TEST / MEASUREMENT INFRASTRUCTURE).
//
// Used only by bench.py's CPU-baseline leg and `bench.py --impl reference`
// to time the reference algorithm on the host cores (OpenMP), and by a test
// that cross-checks it against the numpy oracle.  Never linked into the
// product.  It restates, in float32 arithmetic with float64 scalars:
//   cons/mgpbd_gpu.py:136-151 rest shape; :206-219 prediction/velocity;
//   :225-247 + cons/mgpbd.py:35-68 ARAP C and gradient; :253-267 residual;
//   :273-309 matrix fill on the diagonal-last pattern; :330-355 scatter and
//   apply; :360-391 line search; cons/mgpcg_gpu.py:183-212 coarse refill,
//   :214-259 V-cycle, :261-329 PCG; cons/sparse_gpu.py:107-144 Jacobi.
// The integer structure (pattern, aggregates, coarse pattern, contribution
// map) is passed in from the numpy oracle.  The smoother weight is capped at
// 4/(3 lambda_max(D^-1 A)) per level (power iteration), as in the GPU plain
// arm, because omega = 2/3 diverges on stiff ARAP systems.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Lvl {
  int n = 0;
  std::vector<int32_t> ip, ix;
  std::vector<float> a, dinv;
  float w = 2.0f / 3.0f;
  std::vector<int32_t> agg;                  // -> next level
  std::vector<int32_t> mptr, mrows;          // next level members
  std::vector<int32_t> coff, cidx;           // refill from previous level
  std::vector<float> b, x, x2, r;
  std::vector<float> pw;  // power-iteration vector, kept across Newton iterations
};

struct Cpu {
  int nv, nt;
  std::vector<float> xref, x, v, xold, invm, dpos;
  std::vector<int32_t> t;
  std::vector<float> dminv, alpha, C, g, lam, rhs, dlam;
  std::vector<int32_t> ctype;  // 0 ARAP, 1 length, 2 volume (empty: all ARAP)
  std::vector<float> rest;     // rest length of a length constraint
  std::vector<Lvl> L;
  float dt, mu, compliance, damp, gravity[3];
  int maxiter, maxiter_cg, n_smooth, kinematic;
  double atol, rtol, tol_cg, rel_tol_cg, omega;
  std::vector<float> cr, cz, cp, cap;
};

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// eigen-decomposition of symmetric 3x3 (double, cyclic Jacobi)
void eig3(double a[3][3], double v[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) v[i][j] = i == j;
  for (int sweep = 0; sweep < 12; ++sweep) {
    double off = std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]);
    if (off < 1e-30) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (a[p][q] == 0.0) continue;
        double tau = (a[q][q] - a[p][p]) / (2 * a[p][q]);
        double tt = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1 + tau * tau));
        double c = 1 / std::sqrt(1 + tt * tt), s = tt * c;
        for (int k = 0; k < 3; ++k) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
}

// rotation-variant SVD of F (double), s sorted descending, sign of det on s[2]
void svd3(const double F[3][3], double U[3][3], double s[3], double V[3][3]) {
  double M[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) M[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
  double W[3][3];
  eig3(M, W);
  int id[3] = {0, 1, 2};
  std::sort(id, id + 3, [&](int a, int b) { return M[a][a] > M[b][b]; });
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = W[i][id[j]];
  double det = V[0][0] * (V[1][1] * V[2][2] - V[1][2] * V[2][1]) - V[0][1] * (V[1][0] * V[2][2] - V[1][2] * V[2][0]) +
               V[0][2] * (V[1][0] * V[2][1] - V[1][1] * V[2][0]);
  if (det < 0)
    for (int i = 0; i < 3; ++i) V[i][2] = -V[i][2];
  double B[3][3];  // columns b_c = F v_c
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) B[c][r] = F[r][0] * V[0][c] + F[r][1] * V[1][c] + F[r][2] * V[2][c];
  auto nrm = [](double* x) { return std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); };
  double u1[3] = {B[0][0], B[0][1], B[0][2]}, l1 = nrm(u1);
  if (l1 > 1e-300) for (double& e : u1) e /= l1;
  else { u1[0] = 1; u1[1] = u1[2] = 0; l1 = 0; }
  double d = u1[0] * B[1][0] + u1[1] * B[1][1] + u1[2] * B[1][2];
  double u2[3] = {B[1][0] - d * u1[0], B[1][1] - d * u1[1], B[1][2] - d * u1[2]}, l2 = nrm(u2);
  if (l2 > 1e-300) for (double& e : u2) e /= l2;
  else {
    double e[3] = {0, 0, 0};
    int k = std::fabs(u1[0]) <= std::fabs(u1[1]) ? (std::fabs(u1[0]) <= std::fabs(u1[2]) ? 0 : 2) : (std::fabs(u1[1]) <= std::fabs(u1[2]) ? 1 : 2);
    e[k] = 1;
    u2[0] = u1[1] * e[2] - u1[2] * e[1];
    u2[1] = u1[2] * e[0] - u1[0] * e[2];
    u2[2] = u1[0] * e[1] - u1[1] * e[0];
    double l = nrm(u2);
    for (double& q : u2) q /= l;
  }
  double u3[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2], u1[0] * u2[1] - u1[1] * u2[0]};
  s[0] = l1;
  s[1] = u2[0] * B[1][0] + u2[1] * B[1][1] + u2[2] * B[1][2];
  s[2] = u3[0] * B[2][0] + u3[1] * B[2][1] + u3[2] * B[2][2];
  for (int r = 0; r < 3; ++r) {
    U[r][0] = u1[r];
    U[r][1] = u2[r];
    U[r][2] = u3[r];
  }
}

float arap_c(const Cpu& c, int e, const float* x, const float* dp, float om, double* Ud = nullptr,
             double* sd = nullptr, double* Vd = nullptr) {
  const int32_t* q = &c.t[4 * e];
  float p[4][3];
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k < 3; ++k) p[l][k] = x[3 * q[l] + k] + (dp ? om * dp[3 * q[l] + k] : 0.0f);
  double F[3][3];
  const float* B = &c.dminv[9 * e];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float f = 0;
      for (int k = 0; k < 3; ++k) f += (p[k + 1][i] - p[0][i]) * B[3 * k + j];
      F[i][j] = f;
    }
  double U[3][3], s[3], V[3][3];
  svd3(F, U, s, V);
  float cc = std::sqrt(float((s[0] - 1) * (s[0] - 1) + (s[1] - 1) * (s[1] - 1) + (s[2] - 1) * (s[2] - 1)));
  if (Ud) {
    std::memcpy(Ud, U, sizeof(U));
    std::memcpy(sd, s, sizeof(s));
    std::memcpy(Vd, V, sizeof(V));
  }
  return cc;
}

int ctype_of(const Cpu& c, int e) { return c.ctype.empty() ? 0 : c.ctype[e]; }

// length constraint |x_a - x_b| - L0 (slots 0, 1) and its unit vector a - b
float length_c(const Cpu& c, int e, const float* x, const float* dp, float om, float n[3]) {
  const int32_t* q = &c.t[4 * e];
  float d[3];
  for (int k = 0; k < 3; ++k)
    d[k] = (x[3 * q[0] + k] + (dp ? om * dp[3 * q[0] + k] : 0.0f)) -
           (x[3 * q[1] + k] + (dp ? om * dp[3 * q[1] + k] : 0.0f));
  float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (n)
    for (int k = 0; k < 3; ++k) n[k] = len > 1e-12f ? d[k] / len : 0.0f;
  return len - c.rest[e];
}

// volume constraint det F - 1 and d(det F)/dF (columns f2 x f3, f3 x f1, f1 x f2)
float volume_c(const Cpu& c, int e, const float* x, const float* dp, float om, float P[3][3]) {
  const int32_t* q = &c.t[4 * e];
  float p[4][3];
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k < 3; ++k) p[l][k] = x[3 * q[l] + k] + (dp ? om * dp[3 * q[l] + k] : 0.0f);
  float F[3][3];
  const float* B = &c.dminv[9 * e];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float f = 0;
      for (int k = 0; k < 3; ++k) f += (p[k + 1][i] - p[0][i]) * B[3 * k + j];
      F[i][j] = f;
    }
  const float* f1c[3] = {&F[0][0], &F[1][0], &F[2][0]};
  float f1[3] = {F[0][0], F[1][0], F[2][0]}, f2[3] = {F[0][1], F[1][1], F[2][1]},
        f3[3] = {F[0][2], F[1][2], F[2][2]};
  (void)f1c;
  float c23[3] = {f2[1] * f3[2] - f2[2] * f3[1], f2[2] * f3[0] - f2[0] * f3[2], f2[0] * f3[1] - f2[1] * f3[0]};
  float c31[3] = {f3[1] * f1[2] - f3[2] * f1[1], f3[2] * f1[0] - f3[0] * f1[2], f3[0] * f1[1] - f3[1] * f1[0]};
  float c12[3] = {f1[1] * f2[2] - f1[2] * f2[1], f1[2] * f2[0] - f1[0] * f2[2], f1[0] * f2[1] - f1[1] * f2[0]};
  if (P)
    for (int r = 0; r < 3; ++r) {
      P[r][0] = c23[r];
      P[r][1] = c31[r];
      P[r][2] = c12[r];
    }
  return f1[0] * c23[0] + f1[1] * c23[1] + f1[2] * c23[2] - 1.0f;
}

float cons_c(const Cpu& c, int e, const float* x, const float* dp, float om) {
  const int ty = ctype_of(c, e);
  if (ty == 1) return length_c(c, e, x, dp, om, nullptr);
  if (ty == 2) return volume_c(c, e, x, dp, om, nullptr);
  return arap_c(c, e, x, dp, om);
}

void constraints(Cpu& c) {
#pragma omp parallel for schedule(static)
  for (int e = 0; e < c.nt; ++e) {
    const int ty = ctype_of(c, e);
    if (ty == 1) {
      float n[3];
      c.C[e] = length_c(c, e, c.x.data(), nullptr, 0.0f, n);
      float* g = &c.g[12 * e];
      std::fill(g, g + 12, 0.0f);
      for (int k = 0; k < 3; ++k) {
        g[k] = n[k];
        g[3 + k] = -n[k];
      }
      continue;
    }
    if (ty == 2) {
      float P[3][3];
      c.C[e] = volume_c(c, e, c.x.data(), nullptr, 0.0f, P);
      float* g = &c.g[12 * e];
      const float* B = &c.dminv[9 * e];
      for (int l = 1; l < 4; ++l)
        for (int r = 0; r < 3; ++r)
          g[3 * l + r] = B[3 * (l - 1)] * P[r][0] + B[3 * (l - 1) + 1] * P[r][1] + B[3 * (l - 1) + 2] * P[r][2];
      for (int r = 0; r < 3; ++r) g[r] = -(g[3 + r] + g[6 + r] + g[9 + r]);
      continue;
    }
    double U[3][3], s[3], V[3][3];
    float cc = arap_c(c, e, c.x.data(), nullptr, 0.0f, &U[0][0], s, &V[0][0]);
    c.C[e] = cc;
    float* g = &c.g[12 * e];
    if (cc > 1e-6f) {
      float P[3][3];
      for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
          double acc = 0;
          for (int m = 0; m < 3; ++m) acc += U[r][m] * V[k][m] * ((s[m] - 1) / cc);
          P[r][k] = float(acc);
        }
      const float* B = &c.dminv[9 * e];
      for (int l = 1; l < 4; ++l)
        for (int r = 0; r < 3; ++r)
          g[3 * l + r] = B[3 * (l - 1)] * P[r][0] + B[3 * (l - 1) + 1] * P[r][1] + B[3 * (l - 1) + 2] * P[r][2];
      for (int r = 0; r < 3; ++r) g[r] = -(g[3 + r] + g[6 + r] + g[9 + r]);
    } else {
      std::fill(g, g + 12, 0.0f);
    }
  }
}

void fill(Cpu& c) {
  Lvl& A = c.L[0];
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < c.nt; ++i) {
    const int32_t* qi = &c.t[4 * i];
    const float* gi = &c.g[12 * i];
    for (int k = A.ip[i]; k < A.ip[i + 1] - 1; ++k) {
      int j = A.ix[k];
      const int32_t* qj = &c.t[4 * j];
      const float* gj = &c.g[12 * j];
      float off = 0;
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
          if (qi[a] == qj[b])
            off += c.invm[qi[a]] * (gi[3 * a] * gj[3 * b] + gi[3 * a + 1] * gj[3 * b + 1] + gi[3 * a + 2] * gj[3 * b + 2]);
      A.a[k] = off;
    }
    float d = 0;
    for (int a = 0; a < 4; ++a)
      d += c.invm[qi[a]] * (gi[3 * a] * gi[3 * a] + gi[3 * a + 1] * gi[3 * a + 1] + gi[3 * a + 2] * gi[3 * a + 2]);
    d += c.alpha[i];
    A.a[A.ip[i + 1] - 1] = d;
    A.dinv[i] = std::fabs(d) > 1e-30f ? 1.0f / d : 0.0f;
  }
  for (size_t l = 1; l < c.L.size(); ++l) {
    Lvl& Cl = c.L[l];
    const Lvl& F = c.L[l - 1];
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)Cl.ix.size(); ++e) {
      float s = 0;
      for (int k = Cl.coff[e]; k < Cl.coff[e + 1]; ++k) s += F.a[Cl.cidx[k]];
      Cl.a[e] = s;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Cl.n; ++i) {
      float d = 0;
      for (int k = Cl.ip[i]; k < Cl.ip[i + 1]; ++k)
        if (Cl.ix[k] == i) { d = Cl.a[k]; break; }
      Cl.dinv[i] = std::fabs(d) > 1e-30f ? 1.0f / d : 0.0f;
    }
  }
  // smoother weights: power iteration on D^-1 A, six steps per Newton
  // iteration continuing from the previous iteration's vector (as the GPU
  // plain path does: restarting from a smooth vector every time would
  // underestimate lambda_max and make the smoother diverge)
  for (Lvl& l : c.L) {
    std::vector<float>& v = l.pw;
    std::vector<float> w(l.n);
    double lam = 1;
    for (int it = 0; it < 6; ++it) {
      double nn = 0;
#pragma omp parallel for reduction(+ : nn) schedule(static)
      for (int i = 0; i < l.n; ++i) {
        float s = 0;
        for (int k = l.ip[i]; k < l.ip[i + 1]; ++k) s += l.a[k] * v[l.ix[k]];
        w[i] = l.dinv[i] * s;
        nn += double(w[i]) * w[i];
      }
      double vv = 0;
      for (float e : v) vv += double(e) * e;
      lam = std::sqrt(nn / vv);
      float sc = float(1.0 / std::sqrt(nn));
      for (int i = 0; i < l.n; ++i) v[i] = w[i] * sc;
    }
    float safe = float(4.0 / (3.0 * 1.1 * lam));
    l.w = std::min(float(c.omega), safe);
  }
}

void spmv_res(const Lvl& l, const float* b, const float* x, float* r) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < l.n; ++i) {
    float s = 0;
    for (int k = l.ip[i]; k < l.ip[i + 1]; ++k) s += l.a[k] * x[l.ix[k]];
    r[i] = b ? b[i] - s : s;
  }
}

void jacobi(const Lvl& l, const float* b, const float* x, float* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < l.n; ++i) {
    float s = 0;
    for (int k = l.ip[i]; k < l.ip[i + 1]; ++k) s += l.a[k] * x[l.ix[k]];
    y[i] = x[i] + l.w * l.dinv[i] * (b[i] - s);
  }
}

void vcycle(Cpu& c, int li, const float* b, float* out) {
  Lvl& l = c.L[li];
  std::vector<float>& x = l.x;
  std::vector<float>& y = l.x2;
  std::fill(x.begin(), x.end(), 0.0f);
  auto sweeps = [&](int n) {
    for (int s = 0; s < n; ++s) {
      jacobi(l, b, x.data(), y.data());
      std::swap(x, y);
    }
  };
  if (li + 1 == (int)c.L.size()) {
    sweeps(std::min(50, l.n));
  } else {
    sweeps(c.n_smooth);
    spmv_res(l, b, x.data(), l.r.data());
    Lvl& C = c.L[li + 1];
#pragma omp parallel for schedule(static)
    for (int I = 0; I < C.n; ++I) {
      float s = 0;
      for (int k = l.mptr[I]; k < l.mptr[I + 1]; ++k) s += l.r[l.mrows[k]];
      C.b[I] = s;
    }
    std::vector<float> xc(C.n);
    vcycle(c, li + 1, C.b.data(), xc.data());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < l.n; ++i) x[i] += xc[l.agg[i]];
    sweeps(c.n_smooth);
  }
  std::copy(x.begin(), x.end(), out);
}

double dot(const std::vector<float>& a, const std::vector<float>& b) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < (int64_t)a.size(); ++i) s += double(a[i]) * b[i];
  return s;
}

int pcg(Cpu& c, int cg_max) {
  int n = c.nt;
  std::fill(c.dlam.begin(), c.dlam.end(), 0.0f);
  c.cr = c.rhs;
  vcycle(c, 0, c.cr.data(), c.cz.data());
  c.cp = c.cz;
  double rz = dot(c.cr, c.cz), rr0 = dot(c.rhs, c.rhs);
  double tol2 = std::max(c.tol_cg * c.tol_cg, c.rel_tol_cg * c.rel_tol_cg * rr0);
  int it = 0;
  for (int k = 0; k < cg_max; ++k) {
    spmv_res(c.L[0], nullptr, c.cp.data(), c.cap.data());
    double pap = dot(c.cp, c.cap);
    if (std::fabs(pap) < 1e-30) break;
    double al = rz / pap;
    float a = float(al), na = float(-al);
    double rr = 0;
#pragma omp parallel for reduction(+ : rr) schedule(static)
    for (int i = 0; i < n; ++i) {
      c.dlam[i] += a * c.cp[i];
      c.cr[i] += na * c.cap[i];
      rr += double(c.cr[i]) * c.cr[i];
    }
    if (rr < tol2) { it = k + 1; break; }
    vcycle(c, 0, c.cr.data(), c.cz.data());
    double rzn = dot(c.cr, c.cz);
    if (std::fabs(rz) < 1e-30) { it = k + 1; break; }
    float be = float(rzn / rz);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) c.cp[i] = c.cz[i] + be * c.cp[i];
    rz = rzn;
    it = k + 1;
  }
  return it;
}

double dual_norm(Cpu& c, const float* dp, float om) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int e = 0; e < c.nt; ++e) {
    float cc = dp ? cons_c(c, e, c.x.data(), dp, om) : c.C[e];
    double r = -(cc + c.alpha[e] * c.lam[e]);
    s += r * r;
  }
  return std::sqrt(s);
}

}  // namespace

extern "C" {

void* cpu_create(int nv, int nt, const float* xref, const float* x0, const float* invm,
                 const int32_t* t, float dt, float mu, float compliance, float damp,
                 const float* gravity, int maxiter, double atol, double rtol, int maxiter_cg,
                 double tol_cg, double rel_tol_cg, int n_smooth, double omega, int kinematic,
                 const int32_t* ctype) {
  Cpu* c = new Cpu();
  c->nv = nv;
  c->nt = nt;
  c->xref.assign(xref, xref + 3 * nv);
  c->x.assign(x0, x0 + 3 * nv);
  c->v.assign(3 * nv, 0.0f);
  c->xold.assign(3 * nv, 0.0f);
  c->dpos.assign(3 * nv, 0.0f);
  c->invm.assign(invm, invm + nv);
  c->t.assign(t, t + 4 * nt);
  c->dt = dt;
  c->mu = mu;
  c->compliance = compliance;
  c->damp = damp;
  for (int k = 0; k < 3; ++k) c->gravity[k] = gravity[k];
  c->maxiter = maxiter;
  c->atol = atol;
  c->rtol = rtol;
  c->maxiter_cg = maxiter_cg;
  c->tol_cg = tol_cg;
  c->rel_tol_cg = rel_tol_cg;
  c->n_smooth = n_smooth;
  c->omega = omega;
  c->kinematic = kinematic;
  c->dminv.resize(9 * nt);
  c->alpha.resize(nt);
  c->C.resize(nt);
  c->g.resize(12 * nt);
  c->lam.assign(nt, 0.0f);
  c->rhs.resize(nt);
  c->dlam.resize(nt);
  c->cr.resize(nt);
  c->cz.resize(nt);
  c->cp.resize(nt);
  c->cap.resize(nt);
  if (ctype) c->ctype.assign(ctype, ctype + nt);
  c->rest.assign(nt, 0.0f);
  for (int e = 0; e < nt; ++e) {
    const int32_t* q = &t[4 * e];
    if (ctype && ctype[e] == 1) {  // length: rest length, no Dm^-1
      float d[3];
      for (int k = 0; k < 3; ++k) d[k] = xref[3 * q[0] + k] - xref[3 * q[1] + k];
      c->rest[e] = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      std::fill(&c->dminv[9 * e], &c->dminv[9 * e] + 9, 0.0f);
      c->alpha[e] = compliance > 0 ? compliance / (dt * dt) : 1.0f / (mu * dt * dt * c->rest[e]);
      continue;
    }
    double D[3][3];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) D[i][k] = double(xref[3 * q[k + 1] + i]) - xref[3 * q[0] + i];
    double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) - D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                 D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
    double inv[3][3] = {{D[1][1] * D[2][2] - D[1][2] * D[2][1], D[0][2] * D[2][1] - D[0][1] * D[2][2], D[0][1] * D[1][2] - D[0][2] * D[1][1]},
                        {D[1][2] * D[2][0] - D[1][0] * D[2][2], D[0][0] * D[2][2] - D[0][2] * D[2][0], D[0][2] * D[1][0] - D[0][0] * D[1][2]},
                        {D[1][0] * D[2][1] - D[1][1] * D[2][0], D[0][1] * D[2][0] - D[0][0] * D[2][1], D[0][0] * D[1][1] - D[0][1] * D[1][0]}};
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) c->dminv[9 * e + 3 * i + k] = float(inv[i][k] / det);
    float vol = float(std::fabs(det) / 6.0);
    c->alpha[e] = compliance > 0 ? compliance / (dt * dt) : 1.0f / (mu * dt * dt * vol);
  }
  return c;
}

void cpu_destroy(void* h) { delete static_cast<Cpu*>(h); }

// level 0 pattern; then per coarse level l = 1..: agg of level l-1, coarse
// CSR and contribution map.
int cpu_add_level(void* h, int n, const int32_t* ip, const int32_t* ix, int64_t nnz,
                  const int32_t* agg_prev, const int32_t* coff, const int32_t* cidx) {
  Cpu& c = *static_cast<Cpu*>(h);
  Lvl l;
  l.n = n;
  l.ip.assign(ip, ip + n + 1);
  l.ix.assign(ix, ix + nnz);
  l.a.assign(nnz, 0.0f);
  l.dinv.assign(n, 0.0f);
  l.b.assign(n, 0.0f);
  l.x.assign(n, 0.0f);
  l.x2.assign(n, 0.0f);
  l.r.assign(n, 0.0f);
  l.pw.resize(n);
  for (int i = 0; i < n; ++i) {  // the GPU's pseudo-random start vector
    uint32_t hsh = static_cast<uint32_t>(i) * 2654435761u;
    hsh ^= hsh >> 15;
    l.pw[i] = 0.5f + (hsh & 0xffff) * (1.0f / 65536.0f);
  }
  if (!c.L.empty()) {
    Lvl& F = c.L.back();
    F.agg.assign(agg_prev, agg_prev + F.n);
    F.mptr.assign(n + 1, 0);
    for (int i = 0; i < F.n; ++i) F.mptr[F.agg[i] + 1]++;
    for (int I = 0; I < n; ++I) F.mptr[I + 1] += F.mptr[I];
    F.mrows.resize(F.n);
    std::vector<int32_t> cur(F.mptr.begin(), F.mptr.end() - 1);
    for (int i = 0; i < F.n; ++i) F.mrows[cur[F.agg[i]]++] = i;
    l.coff.assign(coff, coff + nnz + 1);
    l.cidx.assign(cidx, cidx + l.coff.back());
  }
  c.L.push_back(std::move(l));
  return 0;
}

void cpu_predict(void* h) {
  Cpu& c = *static_cast<Cpu*>(h);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < c.nv; ++k) {
    for (int d = 0; d < 3; ++d) c.xold[3 * k + d] = c.x[3 * k + d];
    if (c.kinematic && c.invm[k] == 0.0f) continue;
    for (int d = 0; d < 3; ++d) {
      c.v[3 * k + d] = (c.v[3 * k + d] + c.dt * c.gravity[d]) * c.damp;
      c.x[3 * k + d] += c.dt * c.v[3 * k + d];
    }
  }
  std::fill(c.lam.begin(), c.lam.end(), 0.0f);
}

void cpu_update_vel(void* h) {
  Cpu& c = *static_cast<Cpu*>(h);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < 3 * c.nv; ++k) c.v[k] = c.damp * (c.x[k] - c.xold[k]) / c.dt;
}

// One Newton iteration; returns 1 if the loop's stopping test was met
// (nothing done), 0 otherwise.  out[0] residual, out[1] CG iterations,
// out[2] omega, out[3..] seconds of (constraints+rhs, fill+refill, pcg,
// scatter+line search+apply).
int cpu_newton_iteration(void* h, int ite, double* r0, int cg_max, double* out) {
  Cpu& c = *static_cast<Cpu*>(h);
  double t0 = now();
  constraints(c);
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int e = 0; e < c.nt; ++e) {
    float b = -(c.C[e] + c.alpha[e] * c.lam[e]);
    c.rhs[e] = b;
    s += double(b) * b;
  }
  double r = std::sqrt(s);
  if (ite == 0) *r0 = r;
  out[0] = r;
  double t1 = now();
  if (r < c.atol || (*r0 > 1e-12 && r < c.rtol * *r0)) {
    out[3] = t1 - t0;
    return 1;
  }
  fill(c);
  double t2 = now();
  int it = pcg(c, cg_max);
  double t3 = now();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < c.nt; ++e) c.lam[e] += c.dlam[e];
  std::fill(c.dpos.begin(), c.dpos.end(), 0.0f);
  for (int e = 0; e < c.nt; ++e)  // serial tet order (the reference's loop order)
    for (int l = 0; l < 4; ++l) {
      int vtx = c.t[4 * e + l];
      float sc = c.invm[vtx] * c.dlam[e];
      for (int d = 0; d < 3; ++d) c.dpos[3 * vtx + d] += sc * c.g[12 * e + 3 * l + d];
    }
  double cur = dual_norm(c, nullptr, 0.0f);
  double om = 1.0;
  int k = 0;
  for (; k < 10; ++k) {
    if (dual_norm(c, c.dpos.data(), float(om)) < cur) break;
    om *= 0.5;
  }
#pragma omp parallel for schedule(static)
  for (int vtx = 0; vtx < c.nv; ++vtx)
    if (c.invm[vtx] > 0)
      for (int d = 0; d < 3; ++d) c.x[3 * vtx + d] += float(om) * c.dpos[3 * vtx + d];
  double t4 = now();
  out[1] = it;
  out[2] = om;
  out[3] = t1 - t0;
  out[4] = t2 - t1;
  out[5] = t3 - t2;
  out[6] = t4 - t3;
  return 0;
}

void cpu_get_x(void* h, float* x) {
  Cpu& c = *static_cast<Cpu*>(h);
  std::copy(c.x.begin(), c.x.end(), x);
}

int cpu_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
