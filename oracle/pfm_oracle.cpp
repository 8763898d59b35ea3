// CPU oracle for the particle-flow-map time step: a restatement of the reference's Taichi kernels.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// call this library, always as the oracle that results are compared with or as the timed CPU
// baseline, never as the product path.
//
// Parity status: the reference ships no tests or golden vectors and Taichi 1.5.0 cannot be
// installed here, so this oracle is pinned against golden vectors produced by executing the
// reference's own Python kernels and main() loop through a Taichi-semantics shim
// (tests/golden/make_golden.py, oracle/ref_shim/).  Taichi's own code generation (FMA
// contraction, atomic order) is outside that pin.
//
// Semantics followed (paths are relative to the reference project):
//  * every quantity is f32 (3D/taichi_utils.py:5); Python-scope constants such as `dim-2-eps`
//    are formed in double and rounded to f32 (3D/taichi_utils.py:282-284);
//  * int() truncates toward zero; sample() clamps indices (3D/taichi_utils.py:48-54);
//  * expression evaluation order follows the Python source left to right, without FMA
//    (built with -ffp-contract=off);
//  * struct-for atomics are serialised in index order (particle order for P2G, cell order for
//    the reductions); the restriction scatter is evaluated as the equivalent child-ordered gather.
//
// Layouts are Taichi's: particle vector fields AoS [P][n], grids C-order with the last index
// fastest, face grids padded by one along their own axis (3D/run_3D.py:73-75).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kEps = 1e-6;  // 3D/taichi_utils.py:4

template <class R>
inline R N2(R x) {  // 3D/taichi_utils.py:252-260
  R result = R(0);
  R ax = std::fabs(x);
  if (ax < R(0.5))
    result = R(0.75) - ax * ax;
  else if (ax < R(1.5))
    result = R(0.5) * ((R(1.5) - ax) * (R(1.5) - ax));
  return result;
}

template <class R>
inline R dN2(R x) {  // 3D/taichi_utils.py:262-272
  R result = R(0);
  R ax = std::fabs(x);
  if (ax < R(0.5))
    result = R(-2) * ax;
  else if (ax < R(1.5))
    result = R(0.5) * (R(2) * ax - R(3));
  if (x < R(0)) result *= R(-1);
  return result;
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// --------------------------------------------------------------------------------------------
// 3D grid access
// --------------------------------------------------------------------------------------------
template <class R>
struct Grid3 {
  const R* d;
  int n0, n1, n2;
  inline R at(int i, int j, int k) const { return d[((size_t)i * n1 + j) * n2 + k]; }
  // sample(): int() truncation then clamp (3D/taichi_utils.py:48-54)
  inline R sample(R u, R v, R w) const {
    int i = clampi((int)u, 0, n0 - 1), j = clampi((int)v, 0, n1 - 1), k = clampi((int)w, 0, n2 - 1);
    return at(i, j, k);
  }
};

template <class R>
struct G2Res {
  R val, gx, gy, gz;
};

// interp_grad_2: 3D/taichi_utils.py:275-307
template <class R>
inline G2Res<R> interp_grad_2_3(const Grid3<R>& vf, const R p[3], double dx, R BLx, R BLy, R BLz) {
  const R dxr = R(dx), inv_dx = R(1.0 / dx);
  R u = p[0] / dxr, v = p[1] / dxr, w = p[2] / dxr;
  u = u - BLx; v = v - BLy; w = w - BLz;
  R s = std::max(R(1), std::min(u, R(vf.n0 - 2 - kEps)));
  R t = std::max(R(1), std::min(v, R(vf.n1 - 2 - kEps)));
  R l = std::max(R(1), std::min(w, R(vf.n2 - 2 - kEps)));
  R iu = std::floor(s), iv = std::floor(t), iw = std::floor(l);
  R px = 0, py = 0, pz = 0, interped = 0;
  for (int i = -1; i < 3; ++i)
    for (int j = -1; j < 3; ++j)
      for (int k = -1; k < 3; ++k) {
        R xi = s - (iu + R(i)), yj = t - (iv + R(j)), zk = l - (iw + R(k));
        R value = vf.sample(iu + R(i), iv + R(j), iw + R(k));
        px += inv_dx * (value * dN2(xi) * N2(yj) * N2(zk));
        py += inv_dx * (value * N2(xi) * dN2(yj) * N2(zk));
        pz += inv_dx * (value * N2(xi) * N2(yj) * dN2(zk));
        interped += value * N2(xi) * N2(yj) * N2(zk);
      }
  return {interped, px, py, pz};
}

// interp_grad_2_imp: 3D/taichi_utils.py:327-368 (value, gradient, and new_C = sum dw * value)
template <class R>
inline void interp_grad_2_imp_3(const Grid3<R>& vf, const R p[3], double dx, R BLx, R BLy, R BLz,
                                R* val, R grad[3], R C[3]) {
  const R dxr = R(dx), inv_dx = R(1.0 / dx);
  R u = p[0] / dxr, v = p[1] / dxr, w = p[2] / dxr;
  u = u - BLx; v = v - BLy; w = w - BLz;
  R s = std::max(R(1), std::min(u, R(vf.n0 - 2 - kEps)));
  R t = std::max(R(1), std::min(v, R(vf.n1 - 2 - kEps)));
  R l = std::max(R(1), std::min(w, R(vf.n2 - 2 - kEps)));
  R iu = std::floor(s), iv = std::floor(t), iw = std::floor(l);
  R px = 0, py = 0, pz = 0, interped = 0, c0 = 0, c1 = 0, c2 = 0;
  for (int i = -1; i < 3; ++i)
    for (int j = -1; j < 3; ++j)
      for (int k = -1; k < 3; ++k) {
        R xi = s - (iu + R(i)), yj = t - (iv + R(j)), zk = l - (iw + R(k));
        R value = vf.sample(iu + R(i), iv + R(j), iw + R(k));
        R dwx = inv_dx * dN2(xi) * N2(yj) * N2(zk);
        R dwy = inv_dx * N2(xi) * dN2(yj) * N2(zk);
        R dwz = inv_dx * N2(xi) * N2(yj) * dN2(zk);
        px += value * dwx;
        py += value * dwy;
        pz += value * dwz;
        interped += value * N2(xi) * N2(yj) * N2(zk);
        c0 += dwx * value;
        c1 += dwy * value;
        c2 += dwz * value;
      }
  *val = interped;
  grad[0] = px; grad[1] = py; grad[2] = pz;
  C[0] = c0; C[1] = c1; C[2] = c2;
}

// interp_u_MAC_grad (rows) / _transpose (cols): 3D/taichi_utils.py:312-324.
// g[r][c]: rows form -> g[c][:] = grad(u_c); transpose form -> g[:][c] = grad(u_c).
template <class R>
inline void interp_u_MAC_grad_3(const Grid3<R> u[3], const R p[3], double dx, R uo[3], R g[3][3],
                                bool transpose) {
  const R BL[3][3] = {{R(0), R(0.5), R(0.5)}, {R(0.5), R(0), R(0.5)}, {R(0.5), R(0.5), R(0)}};
  for (int c = 0; c < 3; ++c) {
    G2Res<R> r = interp_grad_2_3(u[c], p, dx, BL[c][0], BL[c][1], BL[c][2]);
    uo[c] = r.val;
    R gr[3] = {r.gx, r.gy, r.gz};
    for (int q = 0; q < 3; ++q) {
      if (transpose)
        g[q][c] = gr[q];
      else
        g[c][q] = gr[q];
    }
  }
}

template <class R>
inline void matvec3(const R M[3][3], const R v[3], R out[3]) {
  for (int r = 0; r < 3; ++r) out[r] = M[r][0] * v[0] + M[r][1] * v[1] + M[r][2] * v[2];
}

template <class R>
inline void matmul3(const R A[3][3], const R B[3][3], R out[3][3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[r][c] = A[r][0] * B[0][c] + A[r][1] * B[1][c] + A[r][2] * B[2][c];
}

// --------------------------------------------------------------------------------------------
// 2D grid access and interpolation (2D/taichi_utils.py)
// --------------------------------------------------------------------------------------------
template <class R>
struct Grid2 {
  const R* d;
  int n0, n1;
  inline R at(int i, int j) const { return d[(size_t)i * n1 + j]; }
  inline R sample(R u, R v) const {  // 2D/taichi_utils.py:23-28
    int i = clampi((int)u, 0, n0 - 1), j = clampi((int)v, 0, n1 - 1);
    return at(i, j);
  }
};

// interp_grad_2 (2D/taichi_utils.py:214-248); the dead new_C accumulation is omitted.
template <class R>
inline void interp_grad_2_2(const Grid2<R>& vf, const R p[2], double dx, R BLx, R BLy, R* val, R grad[2]) {
  const R dxr = R(dx), inv_dx = R(1.0 / dx);
  R u = p[0] / dxr, v = p[1] / dxr;
  u = u - BLx; v = v - BLy;
  R s = std::max(R(1), std::min(u, R(vf.n0 - 2 - kEps)));
  R t = std::max(R(1), std::min(v, R(vf.n1 - 2 - kEps)));
  R iu = std::floor(s), iv = std::floor(t);
  R px = 0, py = 0, interped = 0;
  for (int i = -1; i < 3; ++i)
    for (int j = -1; j < 3; ++j) {
      R xi = s - (iu + R(i)), yj = t - (iv + R(j));
      R value = vf.sample(iu + R(i), iv + R(j));
      px += inv_dx * (value * dN2(xi) * N2(yj));
      py += inv_dx * (value * N2(xi) * dN2(yj));
      interped += value * N2(xi) * N2(yj);
    }
  *val = interped;
  grad[0] = px; grad[1] = py;
}

// interp_grad_2_imp (2D/taichi_utils.py:263-304)
template <class R>
inline void interp_grad_2_imp_2(const Grid2<R>& vf, const R p[2], double dx, R BLx, R BLy, R* val,
                                R grad[2], R C[2]) {
  const R dxr = R(dx), inv_dx = R(1.0 / dx);
  R u = p[0] / dxr, v = p[1] / dxr;
  u = u - BLx; v = v - BLy;
  R s = std::max(R(1), std::min(u, R(vf.n0 - 2 - kEps)));
  R t = std::max(R(1), std::min(v, R(vf.n1 - 2 - kEps)));
  R iu = std::floor(s), iv = std::floor(t);
  R px = 0, py = 0, interped = 0, c0 = 0, c1 = 0;
  for (int i = -1; i < 3; ++i)
    for (int j = -1; j < 3; ++j) {
      R xi = s - (iu + R(i)), yj = t - (iv + R(j));
      R value = vf.sample(iu + R(i), iv + R(j));
      R dwx = inv_dx * dN2(xi) * N2(yj);
      R dwy = inv_dx * N2(xi) * dN2(yj);
      px += value * dwx;
      py += value * dwy;
      interped += value * N2(xi) * N2(yj);
      c0 += dwx * value;
      c1 += dwy * value;
    }
  *val = interped;
  grad[0] = px; grad[1] = py;
  C[0] = c0; C[1] = c1;
}

// interp_u_MAC_grad 2D (2D/taichi_utils.py:257-261): rows form g[c][:] = grad(u_c)
template <class R>
inline void interp_u_MAC_grad_2(const Grid2<R> u[2], const R p[2], double dx, R uo[2], R g[2][2]) {
  const R BL[2][2] = {{R(0), R(0.5)}, {R(0.5), R(0)}};
  for (int c = 0; c < 2; ++c) {
    R gr[2];
    interp_grad_2_2(u[c], p, dx, BL[c][0], BL[c][1], &uo[c], gr);
    g[c][0] = gr[0]; g[c][1] = gr[1];
  }
}

// --------------------------------------------------------------------------------------------
// MGPCG (3D/mgpcg.py:7-280, 350-430; 2D/mgpcg.py:283-365), dimension-generic over a box grid
// --------------------------------------------------------------------------------------------
template <class R>
struct MG {
  int dim;
  int L;
  int bt[3][2];
  std::vector<std::array<int, 3>> dims;
  std::vector<std::vector<R>> r, z;
  std::vector<R> x, p, Ap;
  size_t n0;
  int pre_post = 2, bottom = 50;

  size_t count(int l) const { return (size_t)dims[l][0] * dims[l][1] * (dim == 3 ? dims[l][2] : 1); }

  void setup(int dim_, const int* N, int base_level, const int* boundary, int levels_override) {
    dim = dim_;
    int mn = N[0];
    for (int d = 1; d < dim; ++d) mn = std::min(mn, N[d]);
    L = (int)std::log2((double)mn) - base_level + 1;  // mgpcg.py:28
    if (levels_override > 0) L = levels_override;
    for (int d = 0; d < 3; ++d)
      for (int s = 0; s < 2; ++s) bt[d][s] = (d < dim) ? boundary[d * 2 + s] : 2;
    dims.clear();
    for (int l = 0; l < L; ++l) {
      std::array<int, 3> a{1, 1, 1};
      for (int d = 0; d < dim; ++d) a[d] = N[d] >> l;
      dims.push_back(a);
    }
    r.assign(L, {});
    z.assign(L, {});
    for (int l = 0; l < L; ++l) {
      r[l].assign(count(l), R(0));
      z[l].assign(count(l), R(0));
    }
    n0 = count(0);
    x.assign(n0, R(0));
    p.assign(n0, R(0));
    Ap.assign(n0, R(0));
  }

  inline size_t idx(int l, int i, int j, int k) const {
    return ((size_t)i * dims[l][1] + j) * (dim == 3 ? dims[l][2] : 1) + (dim == 3 ? k : 0);
  }

  // neighbor_sum (mgpcg.py:92-104) and num_fluid_neighbors (mgpcg.py:106-115)
  inline R nbsum(int l, const R* f, int i, int j, int k) const {
    const auto& D = dims[l];
    R ret = R(0);
    int I[3] = {i, j, k};
    for (int d = 0; d < dim; ++d) {
      int Jp[3] = {i, j, k}, Jm[3] = {i, j, k};
      Jp[d] += 1;
      Jm[d] -= 1;
      if (I[d] < D[d] - 1) ret += f[idx(l, Jp[0], Jp[1], Jp[2])];
      if (I[d] > 0) ret += f[idx(l, Jm[0], Jm[1], Jm[2])];
    }
    return ret;
  }
  inline R mult(int l, int i, int j, int k) const {
    const auto& D = dims[l];
    R num = R(2.0 * dim);
    int I[3] = {i, j, k};
    for (int d = 0; d < dim; ++d) {
      if (I[d] <= 0 && bt[d][0] == 2) num -= R(1);
      if (I[d] >= D[d] - 1 && bt[d][1] == 2) num -= R(1);
    }
    return num;
  }

  template <class F>
  void for_cells(int l, F&& f, bool parallel) const {
    const auto& D = dims[l];
    int nk = dim == 3 ? D[2] : 1;
    if (parallel) {
#pragma omp parallel for collapse(2) schedule(static)
      for (int i = 0; i < D[0]; ++i)
        for (int j = 0; j < D[1]; ++j)
          for (int k = 0; k < nk; ++k) f(i, j, k);
    } else {
      for (int i = 0; i < D[0]; ++i)
        for (int j = 0; j < D[1]; ++j)
          for (int k = 0; k < nk; ++k) f(i, j, k);
    }
  }

  void smooth(int l, int phase) {  // mgpcg.py:165-172
    R* zl = z[l].data();
    const R* rl = r[l].data();
    for_cells(l, [&](int i, int j, int k) {
      if (((i + j + k) & 1) == phase) {
        R m = mult(l, i, j, k);
        zl[idx(l, i, j, k)] = (rl[idx(l, i, j, k)] + nbsum(l, zl, i, j, k)) / m;
      }
    }, true);
  }

  void restrict_(int l) {  // mgpcg.py:152-158, as the child-ordered gather of the scatter
    const R* zl = z[l].data();
    const R* rl = r[l].data();
    R* rc = r[l + 1].data();
    const auto& Dc = dims[l + 1];
    const auto& Df = dims[l];
    const R scale_den = R(dim - 1.0);
    int nkc = dim == 3 ? Dc[2] : 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int I = 0; I < Dc[0]; ++I)
      for (int J = 0; J < Dc[1]; ++J)
        for (int K = 0; K < nkc; ++K) {
          R acc = R(0);
          for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
              for (int c = 0; c < (dim == 3 ? 2 : 1); ++c) {
                int i = 2 * I + a, j = 2 * J + b, k = dim == 3 ? 2 * K + c : 0;
                if (i >= Df[0] || j >= Df[1] || (dim == 3 && k >= Df[2])) continue;
                R m = mult(l, i, j, k);
                R res = rl[idx(l, i, j, k)] - (m * zl[idx(l, i, j, k)] - nbsum(l, zl, i, j, k));
                acc += res * R(1.0) / scale_den;
              }
          rc[idx(l + 1, I, J, K)] = acc;
        }
  }

  void prolongate(int l) {  // mgpcg.py:160-163
    R* zl = z[l].data();
    const R* zc = z[l + 1].data();
    for_cells(l, [&](int i, int j, int k) {
      zl[idx(l, i, j, k)] += zc[idx(l + 1, i / 2, j / 2, dim == 3 ? k / 2 : 0)];
    }, true);
  }

  void apply_preconditioner() {  // mgpcg.py:182-200
    std::fill(z[0].begin(), z[0].end(), R(0));
    for (int l = 0; l < L - 1; ++l) {
      for (int s = 0; s < pre_post; ++s) {
        smooth(l, 0);
        smooth(l, 1);
      }
      std::fill(z[l + 1].begin(), z[l + 1].end(), R(0));
      std::fill(r[l + 1].begin(), r[l + 1].end(), R(0));
      restrict_(l);
    }
    for (int s = 0; s < bottom; ++s) {
      smooth(L - 1, 0);
      smooth(L - 1, 1);
    }
    for (int l = L - 2; l >= 0; --l) {
      prolongate(l);
      for (int s = 0; s < pre_post; ++s) {
        smooth(l, 1);
        smooth(l, 0);
      }
    }
  }

  R reduce(const R* a, const R* b) const {  // mgpcg.py:131-135: index-ordered f32 accumulation
    R s = R(0);
    for (size_t q = 0; q < n0; ++q) s += a[q] * b[q];
    return s;
  }

  void recenter(R* rr) const {  // mgpcg.py:174-180
    R mean = R(0);
    const R ne = R((double)n0);
    for (size_t q = 0; q < n0; ++q) mean += rr[q] / ne;
    for (size_t q = 0; q < n0; ++q) rr[q] -= mean;
  }

  void compute_Ap() {  // mgpcg.py:117-122
    const R* pp = p.data();
    R* ap = Ap.data();
    for_cells(0, [&](int i, int j, int k) {
      R m = mult(0, i, j, k);
      ap[idx(0, i, j, k)] = m * pp[idx(0, i, j, k)] - nbsum(0, pp, i, j, k);
    }, true);
  }

  // solve(max_iters, eps, tol): mgpcg.py:202-280.  Returns the iteration reported by the
  // reference's print (it at convergence), or -max_iters when it returns without converging.
  // tol_mode 0: the reference's r.r < tol; 1: |r| < tol |r0| with r0 the recentred initial residual
  // (an exactly zero residual also stops: a zero right-hand side).
  int solve(int max_iters, double eps, double tol, double* final_rTr, int tol_mode = 0, double beta_in = 0.0) {
    bool all_neumann = true;
    for (int d = 0; d < dim; ++d)
      for (int s = 0; s < 2; ++s) all_neumann &= (bt[d][s] == 2);
    R beta = R(beta_in);
    if (all_neumann) recenter(r[0].data());
    double rTr0 = 0.0;
    for (size_t q = 0; q < n0; ++q) rTr0 += (double)r[0][q] * (double)r[0][q];
    apply_preconditioner();
    for (size_t q = 0; q < n0; ++q) p[q] = z[0][q] + beta * p[q];  // update_p
    double old_zTr = (double)reduce(z[0].data(), r[0].data());
    int it = 0;
    double rTr = 0;
    while (max_iters == -1 || it < max_iters) {
      compute_Ap();
      double pAp = (double)reduce(p.data(), Ap.data());
      R alpha = R(old_zTr / (pAp + eps));
      for (size_t q = 0; q < n0; ++q) x[q] += alpha * p[q];
      for (size_t q = 0; q < n0; ++q) r[0][q] -= alpha * Ap[q];
      rTr = (double)reduce(r[0].data(), r[0].data());
      bool stop = tol_mode == 0 ? (rTr < tol) : (rTr == 0.0 || std::sqrt(rTr) < tol * std::sqrt(rTr0));
      if (stop) {
        *final_rTr = rTr;
        return it;
      }
      if (all_neumann) recenter(r[0].data());
      apply_preconditioner();
      double new_zTr = (double)reduce(z[0].data(), r[0].data());
      beta = R(new_zTr / (old_zTr + eps));
      for (size_t q = 0; q < n0; ++q) p[q] = z[0][q] + beta * p[q];
      old_zTr = new_zTr;
      it += 1;
    }
    *final_rTr = rTr;
    return -it;
  }
};

// Poisson(): apply_bc, divergence, init(-div), solve, get_result, subtract_grad_p, apply_bc.
// 3D: mgpcg.py:359-430.
template <class R>
int poisson3(R* ux, R* uy, R* uz, R* p_out, const int* N, int base_level, const int* bt,
             int levels_override, int max_iters, double tol, double* final_rTr, int tol_mode) {
  const int nx = N[0], ny = N[1], nz = N[2];
  auto IX = [&](int i, int j, int k) { return ((size_t)i * ny + j) * nz + k; };
  auto IY = [&](int i, int j, int k) { return ((size_t)i * (ny + 1) + j) * nz + k; };
  auto IZ = [&](int i, int j, int k) { return ((size_t)i * ny + j) * (nz + 1) + k; };
  auto apply_bc = [&]() {
    for (int i = 0; i <= nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
          if (i == 0 && bt[0] == 2) ux[IX(i, j, k)] = 0;
          if (i == nx && bt[1] == 2) ux[IX(i, j, k)] = 0;
        }
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j <= ny; ++j)
        for (int k = 0; k < nz; ++k) {
          if (j == 0 && bt[2] == 2) uy[IY(i, j, k)] = 0;
          if (j == ny && bt[3] == 2) uy[IY(i, j, k)] = 0;
        }
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j)
        for (int k = 0; k <= nz; ++k) {
          if (k == 0 && bt[4] == 2) uz[IZ(i, j, k)] = 0;
          if (k == nz && bt[5] == 2) uz[IZ(i, j, k)] = 0;
        }
  };
  apply_bc();
  MG<R> mg;
  mg.setup(3, N, base_level, bt, levels_override);
  // divergence (mgpcg.py:380-390) and init(u_div, -1) (mgpcg.py:71-79)
#pragma omp parallel for collapse(2)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        R vl = ux[IX(i, j, k)], vr = ux[IX(i + 1, j, k)];
        R vb = uy[IY(i, j, k)], vt = uy[IY(i, j + 1, k)];
        R va = uz[IZ(i, j, k)], vc = uz[IZ(i, j, k + 1)];
        R div = vr - vl + vt - vb + vc - va;
        mg.r[0][mg.idx(0, i, j, k)] = div * R(-1);
      }
  int it = mg.solve(max_iters, 1e-12, tol, final_rTr, tol_mode);
  const R* P = mg.x.data();
  if (p_out) std::memcpy(p_out, P, sizeof(R) * mg.n0);
  auto PI = [&](int i, int j, int k) { return P[((size_t)i * ny + j) * nz + k]; };
  // subtract_grad_p (mgpcg.py:392-418): sample() clamps, then the explicit boundary zeros
#pragma omp parallel for collapse(2)
  for (int i = 0; i <= nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        R pr = PI(clampi(i, 0, nx - 1), j, k), pl = PI(clampi(i - 1, 0, nx - 1), j, k);
        if (i - 1 < 0) pl = 0;
        if (i >= nx) pr = 0;
        ux[IX(i, j, k)] -= (pr - pl);
      }
#pragma omp parallel for collapse(2)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j <= ny; ++j)
      for (int k = 0; k < nz; ++k) {
        R pt = PI(i, clampi(j, 0, ny - 1), k), pb = PI(i, clampi(j - 1, 0, ny - 1), k);
        if (j - 1 < 0) pb = 0;
        if (j >= ny) pt = 0;
        uy[IY(i, j, k)] -= pt - pb;
      }
#pragma omp parallel for collapse(2)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k <= nz; ++k) {
        R pc = PI(i, j, clampi(k, 0, nz - 1)), pa = PI(i, j, clampi(k - 1, 0, nz - 1));
        if (k - 1 < 0) pa = 0;
        if (k >= nz) pc = 0;
        uz[IZ(i, j, k)] -= pc - pa;
      }
  apply_bc();
  return it;
}

// 2D Poisson: 2D/mgpcg.py:293-347
template <class R>
int poisson2(R* ux, R* uy, R* p_out, const int* N, int base_level, const int* bt, int levels_override,
             int max_iters, double tol, double* final_rTr, int tol_mode) {
  const int nx = N[0], ny = N[1];
  auto IX = [&](int i, int j) { return (size_t)i * ny + j; };
  auto IY = [&](int i, int j) { return (size_t)i * (ny + 1) + j; };
  auto apply_bc = [&]() {
    for (int i = 0; i <= nx; ++i)
      for (int j = 0; j < ny; ++j) {
        if (i == 0 && bt[0] == 2) ux[IX(i, j)] = 0;
        if (i == nx && bt[1] == 2) ux[IX(i, j)] = 0;
      }
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j <= ny; ++j) {
        if (j == 0 && bt[2] == 2) uy[IY(i, j)] = 0;
        if (j == ny && bt[3] == 2) uy[IY(i, j)] = 0;
      }
  };
  apply_bc();
  MG<R> mg;
  mg.setup(2, N, base_level, bt, levels_override);
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      R vl = ux[IX(i, j)], vr = ux[IX(i + 1, j)];
      R vb = uy[IY(i, j)], vt = uy[IY(i, j + 1)];
      R div = vr - vl + vt - vb;
      mg.r[0][mg.idx(0, i, j, 0)] = div * R(-1);
    }
  int it = mg.solve(max_iters, 1e-12, tol, final_rTr, tol_mode);
  const R* P = mg.x.data();
  if (p_out) std::memcpy(p_out, P, sizeof(R) * mg.n0);
  auto PI = [&](int i, int j) { return P[(size_t)i * ny + j]; };
  for (int i = 0; i <= nx; ++i)
    for (int j = 0; j < ny; ++j) {
      R pr = PI(clampi(i, 0, nx - 1), j), pl = PI(clampi(i - 1, 0, nx - 1), j);
      if (i - 1 < 0) pl = 0;
      if (i >= nx) pr = 0;
      ux[IX(i, j)] -= (pr - pl);
    }
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j <= ny; ++j) {
      R pt = PI(i, clampi(j, 0, ny - 1)), pb = PI(i, clampi(j - 1, 0, ny - 1));
      if (j - 1 < 0) pb = 0;
      if (j >= ny) pt = 0;
      uy[IY(i, j)] -= pt - pb;
    }
  apply_bc();
  return it;
}

}  // namespace

// ================================================================================================
// C ABI for ctypes.  All arrays are contiguous f32 (f64 where the name says so) in Taichi layout.
// ================================================================================================
extern "C" {

int oracle_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// calc_max_speed: 3D/run_3D.py:95-103
float oracle3_calc_max_speed(const float* ux, const float* uy, const float* uz, int nx, int ny, int nz) {
  float m = 1.e-3f;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        float u = 0.5f * (ux[((size_t)i * ny + j) * nz + k] + ux[((size_t)(i + 1) * ny + j) * nz + k]);
        float v = 0.5f * (uy[((size_t)i * (ny + 1) + j) * nz + k] + uy[((size_t)i * (ny + 1) + j + 1) * nz + k]);
        float w = 0.5f * (uz[((size_t)i * ny + j) * (nz + 1) + k] + uz[((size_t)i * ny + j) * (nz + 1) + k + 1]);
        float sp = std::sqrt(u * u + v * v + w * w);
        m = std::max(m, sp);
      }
  return m;
}

// calc_max_speed: 2D/run_2D.py:101-108
float oracle2_calc_max_speed(const float* ux, const float* uy, int nx, int ny) {
  float m = 1.e-3f;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      float u = 0.5f * (ux[(size_t)i * ny + j] + ux[(size_t)(i + 1) * ny + j]);
      float v = 0.5f * (uy[(size_t)i * (ny + 1) + j] + uy[(size_t)i * (ny + 1) + j + 1]);
      float sp = std::sqrt(u * u + v * v);
      m = std::max(m, sp);
    }
  return m;
}

// init_particles_imp / init_particles_imp_grad_m: 3D/init_conditions.py:254-273.
// imp [P][3] (may be null), C [P][3][3] as (C_x, C_y, C_z) rows (may be null).
void oracle3_g2p(const float* pos, int P, const float* ux, const float* uy, const float* uz, int nx,
                 int ny, int nz, double dx, float* imp, float* C) {
  Grid3<float> u[3] = {{ux, nx + 1, ny, nz}, {uy, nx, ny + 1, nz}, {uz, nx, ny, nz + 1}};
  const float BL[3][3] = {{0.f, 0.5f, 0.5f}, {0.5f, 0.f, 0.5f}, {0.5f, 0.5f, 0.f}};
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    const float* p = pos + (size_t)q * 3;
    for (int c = 0; c < 3; ++c) {
      float val, g[3], Cc[3];
      interp_grad_2_imp_3(u[c], p, dx, BL[c][0], BL[c][1], BL[c][2], &val, g, Cc);
      if (imp) imp[(size_t)q * 3 + c] = val;
      if (C)
        for (int r = 0; r < 3; ++r) C[(size_t)q * 9 + c * 3 + r] = Cc[r];
    }
  }
}

// RK4_T_forward: 3D/run_3D.py:175-219.  pos [P][3]; T [P][3][3] = (T_x, T_y, T_z) vectors.
void oracle3_rk4_T_forward(float* pos, float* T, int P, const float* ux, const float* uy, const float* uz,
                           int nx, int ny, int nz, double dx, float dt) {
  Grid3<float> u[3] = {{ux, nx + 1, ny, nz}, {uy, nx, ny + 1, nz}, {uz, nx, ny, nz + 1}};
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float* ps = pos + (size_t)q * 3;
    float* Tq = T + (size_t)q * 9;
    float p0[3] = {ps[0], ps[1], ps[2]};
    float T0[3][3];
    for (int v = 0; v < 3; ++v)
      for (int c = 0; c < 3; ++c) T0[v][c] = Tq[v * 3 + c];
    float uk[4][3], dT[4][3][3];
    const float stage_c[3] = {0.5f * dt, 0.5f * dt, 1.0f * dt};
    float pk[3] = {p0[0], p0[1], p0[2]};
    float Tk[3][3];
    std::memcpy(Tk, T0, sizeof(Tk));
    for (int s = 0; s < 4; ++s) {
      float g[3][3];
      interp_u_MAC_grad_3(u, pk, dx, uk[s], g, true);
      for (int v = 0; v < 3; ++v) matvec3(g, Tk[v], dT[s][v]);
      if (s < 3) {
        float cdt = stage_c[s];
        for (int c = 0; c < 3; ++c) pk[c] = p0[c] + cdt * uk[s][c];
        for (int v = 0; v < 3; ++v)
          for (int c = 0; c < 3; ++c) Tk[v][c] = T0[v][c] - cdt * dT[s][v][c];
      }
    }
    const float coef = dt * 1.0f / 6.0f;
    for (int c = 0; c < 3; ++c) {
      float sum = uk[0][c] + 2.0f * uk[1][c] + 2.0f * uk[2][c] + uk[3][c];
      ps[c] = p0[c] + coef * sum;
    }
    for (int v = 0; v < 3; ++v)
      for (int c = 0; c < 3; ++c) {
        float sum = dT[0][v][c] + 2.0f * dT[1][v][c] + 2.0f * dT[2][v][c] + dT[3][v][c];
        Tq[v * 3 + c] = T0[v][c] - coef * sum;
      }
  }
}

// update_T: 3D/run_3D.py:430-439.  T_init <- cols(T_gm) @ cols(T_init), both [P][3][3] vector-major.
void oracle3_update_T(float* T_init, const float* T_gm, int P) {
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float* Ti = T_init + (size_t)q * 9;
    const float* Tg = T_gm + (size_t)q * 9;
    float M[3][3], N[3][3], O[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        M[r][c] = Tg[c * 3 + r];
        N[r][c] = Ti[c * 3 + r];
      }
    matmul3(M, N, O);
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) Ti[c * 3 + r] = O[r][c];
  }
}

// P2G: 3D/run_3D.py:441-552.  Particles are scattered in index order with nthreads == 1; with more
// threads each thread scatters a contiguous particle range into a private grid copy and the
// copies are summed in thread order (a deterministic reordering used by the CPU baseline).
void oracle3_p2g(const float* imp0, const float* pos, const float* T_gm, const float* T_init,
                 const float* initC, int P, float* ux, float* uy, float* uz, float* wx, float* wy,
                 float* wz, int nx, int ny, int nz, double dx, int use_apic, int nthreads) {
  const size_t nfx = (size_t)(nx + 1) * ny * nz, nfy = (size_t)nx * (ny + 1) * nz,
               nfz = (size_t)nx * ny * (nz + 1);
  const float dxr = float(dx);
  auto scatter = [&](int q0, int q1, float* gux, float* guy, float* guz, float* gwx, float* gwy, float* gwz) {
    for (int q = q0; q < q1; ++q) {
      const float* Tg = T_gm + (size_t)q * 9;
      const float* Ti = T_init + (size_t)q * 9;
      const float* Cq = initC + (size_t)q * 9;
      float A[3][3], AT[3][3], Cm[3][3], Tin[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          A[r][c] = Tg[r * 3 + c];   // rows(T_gm)
          AT[r][c] = Tg[c * 3 + r];  // cols(T_gm)
          Cm[r][c] = Cq[r * 3 + c];  // rows(init_C)
          Tin[r][c] = Ti[c * 3 + r]; // cols(T_init)
        }
      float CA[3][3], TCT[3][3], TT[3][3], imp[3];
      matmul3(Cm, A, CA);
      matmul3(AT, CA, TCT);
      matmul3(AT, Tin, TT);
      matvec3(TT, imp0 + (size_t)q * 3, imp);
      float p[3] = {pos[(size_t)q * 3 + 0] / dxr, pos[(size_t)q * 3 + 1] / dxr, pos[(size_t)q * 3 + 2] / dxr};
      for (int fam = 0; fam < 3; ++fam) {
        int base[3];
        for (int d = 0; d < 3; ++d) {
          // pos - 0.5*unit(a) - 0.5*unit(b): two f32 subtractions per component
          float t = p[d];
          for (int e = 0; e < 3; ++e)
            if (e != fam) t = t - (d == e ? 0.5f : 0.0f);
          base[d] = (int)t;
        }
        int lim[3] = {nx, ny, nz};
        float* gu = fam == 0 ? gux : (fam == 1 ? guy : guz);
        float* gw = fam == 0 ? gwx : (fam == 1 ? gwy : gwz);
        int s1 = (fam == 1 ? ny + 1 : ny), s2 = (fam == 2 ? nz + 1 : nz);
        for (int oi = -1; oi < 3; ++oi)
          for (int oj = -1; oj < 3; ++oj)
            for (int ok = -1; ok < 3; ++ok) {
              int f[3] = {base[0] + oi, base[1] + oj, base[2] + ok};
              bool in = true;
              for (int d = 0; d < 3; ++d) {
                int hi = (d == fam) ? lim[d] : lim[d] - 1;
                if (f[d] < 0 || f[d] > hi) in = false;
              }
              if (!in) continue;
              float arg[3], dp[3];
              for (int d = 0; d < 3; ++d) {
                arg[d] = (d == fam) ? (p[d] - float(f[d])) : ((p[d] - float(f[d])) - 0.5f);
                dp[d] = ((d == fam) ? (float(f[d]) - p[d]) : ((float(f[d]) + 0.5f) - p[d])) * dxr;
              }
              float weight = N2(arg[0]) * N2(arg[1]) * N2(arg[2]);
              size_t id = ((size_t)f[0] * s1 + f[1]) * s2 + f[2];
              gw[id] += weight;
              float delta = TCT[fam][0] * dp[0] + TCT[fam][1] * dp[1] + TCT[fam][2] * dp[2];
              if (use_apic)
                gu[id] += (imp[fam] + delta) * weight;
              else
                gu[id] += (imp[fam]) * weight;
            }
      }
    }
  };
  std::fill(ux, ux + nfx, 0.f); std::fill(uy, uy + nfy, 0.f); std::fill(uz, uz + nfz, 0.f);
  std::fill(wx, wx + nfx, 0.f); std::fill(wy, wy + nfy, 0.f); std::fill(wz, wz + nfz, 0.f);
  if (nthreads <= 1) {
    scatter(0, P, ux, uy, uz, wx, wy, wz);
  } else {
    size_t tot = 2 * (nfx + nfy + nfz);
    std::vector<float> priv((size_t)nthreads * tot, 0.f);
#pragma omp parallel for num_threads(nthreads) schedule(static, 1)
    for (int t = 0; t < nthreads; ++t) {
      float* b = priv.data() + (size_t)t * tot;
      int q0 = (int)((long long)P * t / nthreads), q1 = (int)((long long)P * (t + 1) / nthreads);
      scatter(q0, q1, b, b + nfx, b + nfx + nfy, b + nfx + nfy + nfz, b + 2 * nfx + nfy + nfz,
              b + 2 * nfx + 2 * nfy + nfz);
    }
    float* outs[6] = {ux, uy, uz, wx, wy, wz};
    size_t lens[6] = {nfx, nfy, nfz, nfx, nfy, nfz};
    size_t offs[6] = {0, nfx, nfx + nfy, nfx + nfy + nfz, 2 * nfx + nfy + nfz, 2 * nfx + 2 * nfy + nfz};
    for (int g = 0; g < 6; ++g) {
#pragma omp parallel for schedule(static)
      for (long long e = 0; e < (long long)lens[g]; ++e) {
        float acc = 0.f;
        for (int t = 0; t < nthreads; ++t) acc += priv[(size_t)t * tot + offs[g] + e];
        outs[g][e] = acc;
      }
    }
  }
  // normalisation: run_3D.py:530-552 (division)
  auto norm = [](float* u, const float* w, size_t n) {
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < (long long)n; ++e)
      if (w[e] > 0) u[e] /= w[e];
  };
  norm(ux, wx, nfx); norm(uy, wy, nfy); norm(uz, wz, nfz);
}

// get_particles_id_in_every_cell: 3D/run_3D.py:342-351 (counts; the id lists are atomics-ordered)
void oracle3_bin_count(const float* pos, int P, int nx, int ny, int nz, double dx, int* count) {
  const float dxr = float(dx);
  std::fill(count, count + (size_t)nx * ny * nz, 0);
  for (int q = 0; q < P; ++q) {
    int c[3];
    for (int d = 0; d < 3; ++d) c[d] = (int)(pos[(size_t)q * 3 + d] / dxr);
    if (c[0] < 0 || c[0] >= nx || c[1] < 0 || c[1] >= ny || c[2] < 0 || c[2] >= nz) continue;
    count[((size_t)c[0] * ny + c[1]) * nz + c[2]] += 1;
  }
}

// Midpoint grid step for one face family: reset_to_identity_grid + RK4_grid (run_3D.py:106-120,
// 144-173) with dt_half = 0.5*curr_dt, then advect_u (run_3D.py:296-312) from u0.
// psi_out/T_out [F][3] (may be null), u_out [F].
void oracle3_midpoint_family(int fam, const float* ux, const float* uy, const float* uz, int nx, int ny,
                             int nz, double dx, float dt_half, float* psi_out, float* T_out, float* u_out) {
  Grid3<float> u[3] = {{ux, nx + 1, ny, nz}, {uy, nx, ny + 1, nz}, {uz, nx, ny, nz + 1}};
  int n0 = nx + (fam == 0), n1 = ny + (fam == 1), n2 = nz + (fam == 2);
  const float dxr = float(dx);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j)
      for (int k = 0; k < n2; ++k) {
        size_t id = ((size_t)i * n1 + j) * n2 + k;
        // X_x/X_y/X_z coordinate fields (taichi_utils.py:33-46): Vector([i, j+0.5, k+0.5]) * dx
        float X[3] = {float(i), float(j), float(k)};
        for (int d = 0; d < 3; ++d)
          if (d != fam) X[d] = X[d] + 0.5f;
        float p0[3] = {X[0] * dxr, X[1] * dxr, X[2] * dxr};
        float T0[3] = {0.f, 0.f, 0.f};
        T0[fam] = 1.f;
        float neg_dt = -1.0f * dt_half;
        float uk[4][3], dT[4][3];
        float pk[3] = {p0[0], p0[1], p0[2]}, Tk[3] = {T0[0], T0[1], T0[2]};
        const float cs[3] = {0.5f * neg_dt, 0.5f * neg_dt, 1.0f * neg_dt};
        for (int s = 0; s < 4; ++s) {
          float g[3][3];
          interp_u_MAC_grad_3(u, pk, dx, uk[s], g, false);
          matvec3(g, Tk, dT[s]);
          if (s < 3) {
            for (int c = 0; c < 3; ++c) pk[c] = p0[c] + cs[s] * uk[s][c];
            for (int c = 0; c < 3; ++c) Tk[c] = T0[c] + cs[s] * dT[s][c];
          }
        }
        const float coef = neg_dt * 1.0f / 6.0f;
        float pf[3], Tf[3];
        for (int c = 0; c < 3; ++c) {
          pf[c] = p0[c] + coef * (uk[0][c] + 2.0f * uk[1][c] + 2.0f * uk[2][c] + uk[3][c]);
          Tf[c] = T0[c] + coef * (dT[0][c] + 2.0f * dT[1][c] + 2.0f * dT[2][c] + dT[3][c]);
        }
        if (psi_out)
          for (int c = 0; c < 3; ++c) psi_out[id * 3 + c] = pf[c];
        if (T_out)
          for (int c = 0; c < 3; ++c) T_out[id * 3 + c] = Tf[c];
        float ua[3], g[3][3];
        interp_u_MAC_grad_3(u, pf, dx, ua, g, false);
        u_out[id] = Tf[0] * ua[0] + Tf[1] * ua[1] + Tf[2] * ua[2];
      }
}

int oracle3_poisson_f32(float* ux, float* uy, float* uz, float* p_out, const int* N, int base_level,
                        const int* bt, int levels, int max_iters, double tol, double* final_rTr, int tol_mode) {
  return poisson3<float>(ux, uy, uz, p_out, N, base_level, bt, levels, max_iters, tol, final_rTr, tol_mode);
}

int oracle3_poisson_f64(double* ux, double* uy, double* uz, double* p_out, const int* N, int base_level,
                        const int* bt, int levels, int max_iters, double tol, double* final_rTr, int tol_mode) {
  return poisson3<double>(ux, uy, uz, p_out, N, base_level, bt, levels, max_iters, tol, final_rTr, tol_mode);
}

// ------------------------------------------------------------------------------------------------
// 2D kernels
// ------------------------------------------------------------------------------------------------

// init_particles_imp / _grad_m (2D/init_conditions.py:184-210). imp [P][2]; C [P][2][2] rows.
void oracle2_g2p(const float* pos, int P, const float* ux, const float* uy, int nx, int ny, double dx,
                 float* imp, float* C) {
  Grid2<float> u[2] = {{ux, nx + 1, ny}, {uy, nx, ny + 1}};
  const float BL[2][2] = {{0.f, 0.5f}, {0.5f, 0.f}};
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    const float* p = pos + (size_t)q * 2;
    for (int c = 0; c < 2; ++c) {
      float val, g[2], Cc[2];
      interp_grad_2_imp_2(u[c], p, dx, BL[c][0], BL[c][1], &val, g, Cc);
      if (imp) imp[(size_t)q * 2 + c] = val;
      if (C) {
        C[(size_t)q * 4 + c * 2 + 0] = Cc[0];
        C[(size_t)q * 4 + c * 2 + 1] = Cc[1];
      }
    }
  }
}

// RK4_T_forward 2D: 2D/run_2D.py:304-341.  T [P][2][2] (T_x, T_y).
void oracle2_rk4_T_forward(float* pos, float* T, int P, const float* ux, const float* uy, int nx, int ny,
                           double dx, float dt, int advect_psi) {
  Grid2<float> u[2] = {{ux, nx + 1, ny}, {uy, nx, ny + 1}};
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float* ps = pos + (size_t)q * 2;
    float* Tq = T + (size_t)q * 4;
    float p0[2] = {ps[0], ps[1]};
    float T0[2][2] = {{Tq[0], Tq[1]}, {Tq[2], Tq[3]}};
    float uk[4][2], dT[4][2][2];
    const float cs[3] = {0.5f * dt, 0.5f * dt, 1.0f * dt};
    float pk[2] = {p0[0], p0[1]}, Tk[2][2] = {{T0[0][0], T0[0][1]}, {T0[1][0], T0[1][1]}};
    for (int s = 0; s < 4; ++s) {
      float g[2][2];
      interp_u_MAC_grad_2(u, pk, dx, uk[s], g);
      // grad.transpose() @ T_v: (g^T T)[r] = g[0][r]*T[0] + g[1][r]*T[1]
      for (int v = 0; v < 2; ++v)
        for (int r = 0; r < 2; ++r) dT[s][v][r] = g[0][r] * Tk[v][0] + g[1][r] * Tk[v][1];
      if (s < 3) {
        for (int c = 0; c < 2; ++c) pk[c] = p0[c] + cs[s] * uk[s][c];
        for (int v = 0; v < 2; ++v)
          for (int c = 0; c < 2; ++c) Tk[v][c] = T0[v][c] - cs[s] * dT[s][v][c];
      }
    }
    const float coef = dt * 1.0f / 6.0f;
    if (advect_psi)
      for (int c = 0; c < 2; ++c) ps[c] = p0[c] + coef * (uk[0][c] + 2.0f * uk[1][c] + 2.0f * uk[2][c] + uk[3][c]);
    for (int v = 0; v < 2; ++v)
      for (int c = 0; c < 2; ++c)
        Tq[v * 2 + c] = T0[v][c] - coef * (dT[0][v][c] + 2.0f * dT[1][v][c] + 2.0f * dT[2][v][c] + dT[3][v][c]);
  }
}

// update_particles_grad_m (2D/run_2D.py:526-536): C = cols(T) @ (rows(C0) @ rows(T))
void oracle2_update_grad_m(float* C, const float* C0, const float* T, int P) {
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    const float* Tq = T + (size_t)q * 4;
    const float* Cq = C0 + (size_t)q * 4;
    float A[2][2] = {{Tq[0], Tq[1]}, {Tq[2], Tq[3]}};   // rows
    float AT[2][2] = {{Tq[0], Tq[2]}, {Tq[1], Tq[3]}};  // cols
    float Cm[2][2] = {{Cq[0], Cq[1]}, {Cq[2], Cq[3]}};
    float CA[2][2], O[2][2];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) CA[r][c] = Cm[r][0] * A[0][c] + Cm[r][1] * A[1][c];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) O[r][c] = AT[r][0] * CA[0][c] + AT[r][1] * CA[1][c];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) C[(size_t)q * 4 + r * 2 + c] = O[r][c];
  }
}

// update_T 2D (2D/run_2D.py:538-546): T <- cols(T_gm) @ cols(T_init)
void oracle2_update_T(float* T, const float* T_init, const float* T_gm, int P) {
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    const float* G = T_gm + (size_t)q * 4;
    const float* I = T_init + (size_t)q * 4;
    float M[2][2] = {{G[0], G[2]}, {G[1], G[3]}};
    float N[2][2] = {{I[0], I[2]}, {I[1], I[3]}};
    for (int c = 0; c < 2; ++c)
      for (int r = 0; r < 2; ++r) T[(size_t)q * 4 + c * 2 + r] = M[r][0] * N[0][c] + M[r][1] * N[1][c];
  }
}

// update_particles_imp 2D (2D/run_2D.py:517-524): imp = cols(T_x, T_y) @ init_imp
void oracle2_update_imp(float* imp, const float* imp0, const float* T, int P) {
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    const float* Tq = T + (size_t)q * 4;
    const float* m = imp0 + (size_t)q * 2;
    imp[(size_t)q * 2 + 0] = Tq[0] * m[0] + Tq[2] * m[1];
    imp[(size_t)q * 2 + 1] = Tq[1] * m[0] + Tq[3] * m[1];
  }
}

// P2G 2D: 2D/run_2D.py:548-611 (impulse with APIC C, and the reference map psi; scale = 1/w).
void oracle2_p2g(const float* imp, const float* pos, const float* C, const float* psi, int P, float* ux,
                 float* uy, float* psix, float* psiy, float* wx, float* wy, int nx, int ny, double dx,
                 int use_apic) {
  const size_t nfx = (size_t)(nx + 1) * ny, nfy = (size_t)nx * (ny + 1);
  const float dxr = float(dx);
  std::fill(ux, ux + nfx, 0.f); std::fill(uy, uy + nfy, 0.f);
  std::fill(wx, wx + nfx, 0.f); std::fill(wy, wy + nfy, 0.f);
  if (psix) std::fill(psix, psix + 2 * nfx, 0.f);
  if (psiy) std::fill(psiy, psiy + 2 * nfy, 0.f);
  for (int q = 0; q < P; ++q) {
    float p[2] = {pos[(size_t)q * 2] / dxr, pos[(size_t)q * 2 + 1] / dxr};
    for (int fam = 0; fam < 2; ++fam) {
      int base[2];
      if (fam == 0) {
        base[0] = (int)(p[0] - 0.0f);
        base[1] = (int)(p[1] - 0.5f);
      } else {
        base[0] = (int)(p[0] - 0.5f);
        base[1] = (int)(p[1] - 0.0f);
      }
      float* gu = fam == 0 ? ux : uy;
      float* gw = fam == 0 ? wx : wy;
      float* gp = fam == 0 ? psix : psiy;
      int s1 = fam == 1 ? ny + 1 : ny;
      const float* Cq = C + (size_t)q * 4 + fam * 2;
      for (int oi = -1; oi < 3; ++oi)
        for (int oj = -1; oj < 3; ++oj) {
          int f0 = base[0] + oi, f1 = base[1] + oj;
          bool in = fam == 0 ? (0 <= f0 && f0 <= nx && 0 <= f1 && f1 < ny)
                             : (0 <= f0 && f0 < nx && 0 <= f1 && f1 <= ny);
          if (!in) continue;
          float weight, dp0, dp1;
          if (fam == 0) {
            weight = N2(p[0] - float(f0)) * N2((p[1] - float(f1)) - 0.5f);
            dp0 = (float(f0) - p[0]) * dxr;
            dp1 = ((float(f1) + 0.5f) - p[1]) * dxr;
          } else {
            weight = N2((p[0] - float(f0)) - 0.5f) * N2(p[1] - float(f1));
            dp0 = ((float(f0) + 0.5f) - p[0]) * dxr;
            dp1 = (float(f1) - p[1]) * dxr;
          }
          size_t id = (size_t)f0 * s1 + f1;
          gw[id] += weight;
          float delta = Cq[0] * dp0 + Cq[1] * dp1;
          if (use_apic)
            gu[id] += (imp[(size_t)q * 2 + fam] + delta) * weight;
          else
            gu[id] += imp[(size_t)q * 2 + fam] * weight;
          if (gp) {
            gp[id * 2 + 0] += psi[(size_t)q * 2 + 0] * weight;
            gp[id * 2 + 1] += psi[(size_t)q * 2 + 1] * weight;
          }
        }
    }
  }
  for (int fam = 0; fam < 2; ++fam) {
    float* gu = fam == 0 ? ux : uy;
    float* gw = fam == 0 ? wx : wy;
    float* gp = fam == 0 ? psix : psiy;
    size_t n = fam == 0 ? nfx : nfy;
    for (size_t e = 0; e < n; ++e)
      if (gw[e] > 0) {
        float scale = 1.0f / gw[e];
        gu[e] *= scale;
        if (gp) {
          gp[e * 2] *= scale;
          gp[e * 2 + 1] *= scale;
        }
      }
  }
}

// 2D midpoint for one family: reset_to_identity_grid + RK4_grid + advect_u (run_2D.py:120-129,
// 233-261, 429-441).
void oracle2_midpoint_family(int fam, const float* ux, const float* uy, int nx, int ny, double dx,
                             float dt_half, float* psi_out, float* T_out, float* u_out) {
  Grid2<float> u[2] = {{ux, nx + 1, ny}, {uy, nx, ny + 1}};
  int n0 = nx + (fam == 0), n1 = ny + (fam == 1);
  const float dxr = float(dx);
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j) {
      size_t id = (size_t)i * n1 + j;
      // horizontal_coords_func / vertical_coords_func (2D/taichi_utils.py:40-48)
      float X[2] = {float(i), float(j)};
      if (fam == 0) X[1] = X[1] + 0.5f; else X[0] = X[0] + 0.5f;
      float p0[2] = {X[0] * dxr, X[1] * dxr};
      float T0[2] = {fam == 0 ? 1.f : 0.f, fam == 1 ? 1.f : 0.f};
      float neg_dt = -1.0f * dt_half;
      const float cs[3] = {0.5f * neg_dt, 0.5f * neg_dt, 1.0f * neg_dt};
      float uk[4][2], dT[4][2];
      float pk[2] = {p0[0], p0[1]}, Tk[2] = {T0[0], T0[1]};
      for (int s = 0; s < 4; ++s) {
        float g[2][2];
        interp_u_MAC_grad_2(u, pk, dx, uk[s], g);
        for (int r = 0; r < 2; ++r) dT[s][r] = g[r][0] * Tk[0] + g[r][1] * Tk[1];
        if (s < 3) {
          for (int c = 0; c < 2; ++c) pk[c] = p0[c] + cs[s] * uk[s][c];
          for (int c = 0; c < 2; ++c) Tk[c] = T0[c] + cs[s] * dT[s][c];
        }
      }
      const float coef = neg_dt * 1.0f / 6.0f;
      float pf[2], Tf[2];
      for (int c = 0; c < 2; ++c) {
        pf[c] = p0[c] + coef * (uk[0][c] + 2.0f * uk[1][c] + 2.0f * uk[2][c] + uk[3][c]);
        Tf[c] = T0[c] + coef * (dT[0][c] + 2.0f * dT[1][c] + 2.0f * dT[2][c] + dT[3][c]);
      }
      if (psi_out) { psi_out[id * 2] = pf[0]; psi_out[id * 2 + 1] = pf[1]; }
      if (T_out) { T_out[id * 2] = Tf[0]; T_out[id * 2 + 1] = Tf[1]; }
      float ua[2], g[2][2];
      interp_u_MAC_grad_2(u, pf, dx, ua, g);
      u_out[id] = Tf[0] * ua[0] + Tf[1] * ua[1];
    }
}

int oracle2_poisson_f32(float* ux, float* uy, float* p_out, const int* N, int base_level, const int* bt,
                        int levels, int max_iters, double tol, double* final_rTr, int tol_mode) {
  return poisson2<float>(ux, uy, p_out, N, base_level, bt, levels, max_iters, tol, final_rTr, tol_mode);
}

int oracle2_poisson_f64(double* ux, double* uy, double* p_out, const int* N, int base_level, const int* bt,
                        int levels, int max_iters, double tol, double* final_rTr, int tol_mode) {
  return poisson2<double>(ux, uy, p_out, N, base_level, bt, levels, max_iters, tol, final_rTr, tol_mode);
}

// ------------------------------------------------------------------------------------------------
// scalar (smoke) transport and diagnostics
// ------------------------------------------------------------------------------------------------

// get_central_vector (3D/taichi_utils.py:80-85): vc [nx][ny][nz][3]
void oracle3_central_vector(const float* ux, const float* uy, const float* uz, int nx, int ny, int nz, float* vc) {
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        size_t e = ((size_t)i * ny + j) * nz + k;
        vc[e * 3 + 0] = 0.5f * (ux[((size_t)(i + 1) * ny + j) * nz + k] + ux[((size_t)i * ny + j) * nz + k]);
        vc[e * 3 + 1] = 0.5f * (uy[((size_t)i * (ny + 1) + j + 1) * nz + k] + uy[((size_t)i * (ny + 1) + j) * nz + k]);
        vc[e * 3 + 2] = 0.5f * (uz[((size_t)i * ny + j) * (nz + 1) + k + 1] + uz[((size_t)i * ny + j) * (nz + 1) + k]);
      }
}

// curl (3D/taichi_utils.py:56-78): w [nx][ny][nz][3]; sample() clamps the neighbour indices.
void oracle3_curl(const float* vc, int nx, int ny, int nz, float dx, float* w) {
  const float inv_dist = 1.0f / (2.0f * dx);
  auto at = [&](int i, int j, int k, int c) {
    i = clampi(i, 0, nx - 1); j = clampi(j, 0, ny - 1); k = clampi(k, 0, nz - 1);
    return vc[(((size_t)i * ny + j) * nz + k) * 3 + c];
  };
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        float d_vx_dz = inv_dist * (at(i, j, k + 1, 0) - at(i, j, k - 1, 0));
        float d_vx_dy = inv_dist * (at(i, j + 1, k, 0) - at(i, j - 1, k, 0));
        float d_vy_dx = inv_dist * (at(i + 1, j, k, 1) - at(i - 1, j, k, 1));
        float d_vy_dz = inv_dist * (at(i, j, k + 1, 1) - at(i, j, k - 1, 1));
        float d_vz_dx = inv_dist * (at(i + 1, j, k, 2) - at(i - 1, j, k, 2));
        float d_vz_dy = inv_dist * (at(i, j + 1, k, 2) - at(i, j - 1, k, 2));
        size_t e = ((size_t)i * ny + j) * nz + k;
        w[e * 3 + 0] = d_vz_dy - d_vy_dz;
        w[e * 3 + 1] = d_vx_dz - d_vz_dx;
        w[e * 3 + 2] = d_vy_dx - d_vx_dy;
      }
}

// get_central_vector (2D/taichi_utils.py:50-55): vc [nx][ny][2]
void oracle2_central_vector(const float* ux, const float* uy, int nx, int ny, float* vc) {
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      size_t e = (size_t)i * ny + j;
      vc[e * 2 + 0] = 0.5f * (ux[(size_t)(i + 1) * ny + j] + ux[(size_t)i * ny + j]);
      vc[e * 2 + 1] = 0.5f * (uy[(size_t)i * (ny + 1) + j + 1] + uy[(size_t)i * (ny + 1) + j]);
    }
}

// curl (2D/taichi_utils.py:96-104): w [nx][ny] = (vr.y - vl.y - vt.x + vb.x) / (2 dx)
void oracle2_curl(const float* vc, int nx, int ny, float dx, float* w) {
  auto at = [&](int i, int j, int c) {
    i = clampi(i, 0, nx - 1); j = clampi(j, 0, ny - 1);
    return vc[((size_t)i * ny + j) * 2 + c];
  };
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      w[(size_t)i * ny + j] = (at(i + 1, j, 1) - at(i - 1, j, 1) - at(i, j + 1, 0) + at(i, j - 1, 0)) / (2.0f * dx);
}

// init_particles_smoke (3D/init_conditions.py:275-279) with interp_grad_2_smoke
// (3D/taichi_utils.py:379-420), BL = 0.5.  smoke [nx][ny][nz][4]; s_out [P][4]; grad_out [P][3][4].
void oracle3_init_particles_smoke(const float* pos, int P, const float* smoke, int nx, int ny, int nz, float dx,
                                  float* s_out, float* grad_out) {
  const int n[3] = {nx, ny, nz};
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float u[3], st[3], iu[3];
    for (int a = 0; a < 3; ++a) {
      u[a] = pos[(size_t)q * 3 + a] / dx;
      u[a] = u[a] - 0.5f;
      st[a] = std::max(1.0f, std::min(u[a], float(n[a] - 2 - kEps)));
      iu[a] = std::floor(st[a]);
    }
    const float inv = 1.0f / dx;
    float val[4] = {0, 0, 0, 0}, C[3][4] = {{0}};
    for (int i = -1; i < 3; ++i)
      for (int j = -1; j < 3; ++j)
        for (int k = -1; k < 3; ++k) {
          float xi = st[0] - (iu[0] + float(i)), yj = st[1] - (iu[1] + float(j)), zk = st[2] - (iu[2] + float(k));
          int ci = clampi((int)(iu[0] + float(i)), 0, nx - 1), cj = clampi((int)(iu[1] + float(j)), 0, ny - 1),
              ck = clampi((int)(iu[2] + float(k)), 0, nz - 1);
          const float* v = smoke + (((size_t)ci * ny + cj) * nz + ck) * 4;
          float dw[3] = {inv * dN2(xi) * N2(yj) * N2(zk), inv * N2(xi) * dN2(yj) * N2(zk),
                         inv * N2(xi) * N2(yj) * dN2(zk)};
          for (int ch = 0; ch < 4; ++ch) {
            val[ch] += v[ch] * N2(xi) * N2(yj) * N2(zk);
            for (int r = 0; r < 3; ++r) C[r][ch] += dw[r] * v[ch];
          }
        }
    for (int ch = 0; ch < 4; ++ch) {
      if (s_out) s_out[(size_t)q * 4 + ch] = val[ch];
      if (grad_out)
        for (int r = 0; r < 3; ++r) grad_out[(size_t)q * 12 + r * 4 + ch] = C[r][ch];
    }
  }
}

// P2G_smoke (3D/run_3D.py:554-593), particles scattered in index order.  s [P][4],
// G = init_grad_smoke [P][3][4], T_gm/T_init [P][3][3] (x, y, z vectors); smoke [nx][ny][nz][4],
// w [nx][ny][nz].
void oracle3_p2g_smoke(const float* s, const float* G, const float* pos, const float* T_gm, const float* T_init, int P,
                       float* smoke, float* w, int nx, int ny, int nz, double dx, int use_apic) {
  const size_t C = (size_t)nx * ny * nz;
  std::fill(smoke, smoke + C * 4, 0.f);
  std::fill(w, w + C, 0.f);
  const float dxr = float(dx);
  for (int q = 0; q < P; ++q) {
    float AT[3][3], Tin[3][3], TT[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        AT[r][c] = T_gm[(size_t)q * 9 + c * 3 + r];   // cols(T_gm)
        Tin[r][c] = T_init[(size_t)q * 9 + c * 3 + r]; // cols(T_init)
      }
    matmul3(AT, Tin, TT);
    float M[3][4];
    for (int r = 0; r < 3; ++r)
      for (int ch = 0; ch < 4; ++ch)
        M[r][ch] = TT[r][0] * G[(size_t)q * 12 + 0 * 4 + ch] + TT[r][1] * G[(size_t)q * 12 + 1 * 4 + ch] +
                   TT[r][2] * G[(size_t)q * 12 + 2 * 4 + ch];
    float p[3] = {pos[(size_t)q * 3] / dxr, pos[(size_t)q * 3 + 1] / dxr, pos[(size_t)q * 3 + 2] / dxr};
    int base[3] = {(int)(p[0] - 0.5f), (int)(p[1] - 0.5f), (int)(p[2] - 0.5f)};
    for (int oi = -1; oi < 3; ++oi)
      for (int oj = -1; oj < 3; ++oj)
        for (int ok = -1; ok < 3; ++ok) {
          int f[3] = {base[0] + oi, base[1] + oj, base[2] + ok};
          if (!(0 <= f[0] && f[0] < nx && 0 <= f[1] && f[1] < ny && 0 <= f[2] && f[2] < nz)) continue;
          float weight = N2((p[0] - float(f[0])) - 0.5f) * N2((p[1] - float(f[1])) - 0.5f) *
                         N2((p[2] - float(f[2])) - 0.5f);
          float dp[3];
          for (int d = 0; d < 3; ++d) dp[d] = ((float(f[d]) + 0.5f) - p[d]) * dxr;
          size_t id = ((size_t)f[0] * ny + f[1]) * nz + f[2];
          w[id] += weight;
          for (int ch = 0; ch < 4; ++ch) {
            float delta = dp[0] * M[0][ch] + dp[1] * M[1][ch] + dp[2] * M[2][ch];
            float v = s[(size_t)q * 4 + ch];
            smoke[id * 4 + ch] += (use_apic ? (v + delta) : v) * weight;
          }
        }
  }
  for (size_t e = 0; e < C; ++e)
    if (w[e] > 0) {
      for (int ch = 0; ch < 4; ++ch) {
        float x = smoke[e * 4 + ch] / w[e];
        if (x < 0.f) x = 0.f;
        if (x > 1.f) x = 1.f;
        smoke[e * 4 + ch] = x;
      }
    }
}

// advect_smoke (clamp = 0) / clamp_smoke (clamp = 1): 3D/run_3D.py:315-334 with interp_1 /
// sample_min_max_1 (3D/taichi_utils.py:192-250).  smoke [nx][ny][nz][4], psi grids [F][3].
void oracle3_advect_smoke(const float* s0, float* s1, const float* px, const float* py, const float* pz, int nx,
                          int ny, int nz, float dx, int clamp) {
  const int n[3] = {nx, ny, nz};
  const float sixth = float(1.0 / 6.0);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j)
      for (int k = 0; k < nz; ++k) {
        const float* a = px + (((size_t)i * ny + j) * nz + k) * 3;
        const float* b = px + (((size_t)(i + 1) * ny + j) * nz + k) * 3;
        const float* c = py + (((size_t)i * (ny + 1) + j) * nz + k) * 3;
        const float* d = py + (((size_t)i * (ny + 1) + j + 1) * nz + k) * 3;
        const float* e = pz + (((size_t)i * ny + j) * (nz + 1) + k) * 3;
        const float* f = pz + (((size_t)i * ny + j) * (nz + 1) + k + 1) * 3;
        float st[3], iu[3];
        for (int t = 0; t < 3; ++t) {
          float pc = sixth * (a[t] + b[t] + c[t] + d[t] + e[t] + f[t]);
          float u = pc / dx;
          u = u - 0.5f;
          st[t] = std::max(1.0f, std::min(u, float(n[t] - 1 - kEps)));
          iu[t] = std::floor(st[t]);
        }
        auto at = [&](float fi, float fj, float fk) {
          int ci = clampi((int)fi, 0, nx - 1), cj = clampi((int)fj, 0, ny - 1), ck = clampi((int)fk, 0, nz - 1);
          return s0 + (((size_t)ci * ny + cj) * nz + ck) * 4;
        };
        float* out = s1 + (((size_t)i * ny + j) * nz + k) * 4;
        if (!clamp) {
          const float* v0 = at(iu[0], iu[1], iu[2]);
          float acc[4];
          for (int ch = 0; ch < 4; ++ch) acc[ch] = 0.f * v0[ch];
          for (int a2 = 0; a2 < 2; ++a2)
            for (int b2 = 0; b2 < 2; ++b2)
              for (int c2 = 0; c2 < 2; ++c2) {
                float x = st[0] - (iu[0] + float(a2)), y = st[1] - (iu[1] + float(b2)), z = st[2] - (iu[2] + float(c2));
                const float* v = at(iu[0] + float(a2), iu[1] + float(b2), iu[2] + float(c2));
                float nxw = 1.0f - std::fabs(x), nyw = 1.0f - std::fabs(y), nzw = 1.0f - std::fabs(z);
                for (int ch = 0; ch < 4; ++ch) acc[ch] += v[ch] * nxw * nyw * nzw;
              }
          for (int ch = 0; ch < 4; ++ch) out[ch] = acc[ch];
        } else {
          const float* v0 = at(iu[0], iu[1], iu[2]);
          float mn[4], mx[4];
          for (int ch = 0; ch < 4; ++ch) mn[ch] = mx[ch] = v0[ch];
          for (int a2 = 0; a2 < 2; ++a2)
            for (int b2 = 0; b2 < 2; ++b2)
              for (int c2 = 0; c2 < 2; ++c2) {
                const float* v = at(iu[0] + float(a2), iu[1] + float(b2), iu[2] + float(c2));
                for (int ch = 0; ch < 4; ++ch) {
                  mn[ch] = std::min(mn[ch], v[ch]);
                  mx[ch] = std::max(mx[ch], v[ch]);
                }
              }
          for (int ch = 0; ch < 4; ++ch) out[ch] = std::min(std::max(out[ch], mn[ch]), mx[ch]);
        }
      }
}

// advect_smoke (2D/run_2D.py:444-450) with interp_1 (2D/taichi_utils.py:118-143).  smoke [nx][ny][3],
// psi grids [F][2].
void oracle2_advect_smoke(const float* s0, float* s1, const float* px, const float* py, int nx, int ny, float dx) {
  const int n[2] = {nx, ny};
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      const float* a = px + ((size_t)i * ny + j) * 2;
      const float* b = px + ((size_t)(i + 1) * ny + j) * 2;
      const float* c = py + ((size_t)i * (ny + 1) + j) * 2;
      const float* d = py + ((size_t)i * (ny + 1) + j + 1) * 2;
      float st[2], iu[2];
      for (int t = 0; t < 2; ++t) {
        float pc = 0.25f * (a[t] + b[t] + c[t] + d[t]);
        float u = pc / dx;
        u = u - 0.5f;
        st[t] = std::max(0.0f, std::min(u, float(n[t] - 1 - kEps)));
        iu[t] = std::floor(st[t]);
      }
      float fu = st[0] - iu[0], fv = st[1] - iu[1];
      auto at = [&](float fi, float fj) {
        int ci = clampi((int)fi, 0, nx - 1), cj = clampi((int)fj, 0, ny - 1);
        return s0 + ((size_t)ci * ny + cj) * 3;
      };
      const float *va = at(iu[0], iu[1]), *vb = at(iu[0] + 1, iu[1]), *vc = at(iu[0], iu[1] + 1),
                  *vd = at(iu[0] + 1, iu[1] + 1);
      auto N1 = [](float x) { return 1.0f - std::fabs(x); };
      for (int ch = 0; ch < 3; ++ch)
        s1[((size_t)i * ny + j) * 3 + ch] = va[ch] * N1(fu) * N1(fv) + vb[ch] * N1(fu - 1) * N1(fv) +
                                            vc[ch] * N1(fu) * N1(fv - 1) + vd[ch] * N1(fu - 1) * N1(fv - 1);
    }
}

// ------------------------------------------------------------------------------------------------
// the alternative ("evolve m") dataflow: kernels the live step does not call
// ------------------------------------------------------------------------------------------------

// RK4_T_and_T_grad_m_forward: 3D/run_3D.py:221-292.  pos [P][3]; T, T2 [P][3][3] (x, y, z vectors).
void oracle3_rk4_T_and_T_grad_m_forward(float* pos, float* T, float* T2, int P, const float* ux, const float* uy,
                                        const float* uz, int nx, int ny, int nz, double dx, float dt) {
  Grid3<float> u[3] = {{ux, nx + 1, ny, nz}, {uy, nx, ny + 1, nz}, {uz, nx, ny, nz + 1}};
  const float one_sixth = float(1.0 / 6.0);
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float* ps = pos + (size_t)q * 3;
    float* Tq[2] = {T + (size_t)q * 9, T2 + (size_t)q * 9};
    float p0[3] = {ps[0], ps[1], ps[2]};
    float T0[2][3][3];
    for (int s2 = 0; s2 < 2; ++s2)
      for (int v = 0; v < 3; ++v)
        for (int c = 0; c < 3; ++c) T0[s2][v][c] = Tq[s2][v * 3 + c];
    float uk[4][3], dT[4][2][3][3];
    const float half_dt = 0.5f * dt;
    const float stage_c[3] = {half_dt, half_dt, dt};
    float pk[3] = {p0[0], p0[1], p0[2]};
    float Tk[2][3][3];
    std::memcpy(Tk, T0, sizeof(Tk));
    for (int s = 0; s < 4; ++s) {
      float g[3][3];
      interp_u_MAC_grad_3(u, pk, dx, uk[s], g, true);
      for (int s2 = 0; s2 < 2; ++s2)
        for (int v = 0; v < 3; ++v) matvec3(g, Tk[s2][v], dT[s][s2][v]);
      if (s < 3) {
        float cdt = stage_c[s];
        for (int c = 0; c < 3; ++c) pk[c] = p0[c] + cdt * uk[s][c];
        for (int s2 = 0; s2 < 2; ++s2)
          for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c) Tk[s2][v][c] = T0[s2][v][c] - cdt * dT[s][s2][v][c];
      }
    }
    const float coef = dt * one_sixth;
    for (int c = 0; c < 3; ++c) ps[c] = p0[c] + coef * (uk[0][c] + 2.0f * uk[1][c] + 2.0f * uk[2][c] + uk[3][c]);
    for (int s2 = 0; s2 < 2; ++s2)
      for (int v = 0; v < 3; ++v)
        for (int c = 0; c < 3; ++c)
          Tq[s2][v * 3 + c] = T0[s2][v][c] - coef * (dT[0][s2][v][c] + 2.0f * dT[1][s2][v][c] +
                                                     2.0f * dT[2][s2][v][c] + dT[3][s2][v][c]);
  }
}

// update_particles_imp: 3D/run_3D.py:395-401.  imp [P][3] = cols(T) @ init_imp
void oracle3_update_imp(float* imp, const float* imp0, const float* T, int P) {
  for (int q = 0; q < P; ++q) {
    const float* Tq = T + (size_t)q * 9;
    const float* m = imp0 + (size_t)q * 3;
    for (int r = 0; r < 3; ++r) imp[(size_t)q * 3 + r] = Tq[0 * 3 + r] * m[0] + Tq[1 * 3 + r] * m[1] + Tq[2 * 3 + r] * m[2];
  }
}

// update_particles_grad_m: 3D/run_3D.py:412-428.  C, C0 [P][3][3] rows; T [P][3][3];
// gT [P][3][3][3] (grad_T_init_x/y/z matrices, may be null); imp0 [P][3].
void oracle3_update_grad_m(float* C, const float* C0, const float* T, const float* gT, const float* imp0, int P) {
  for (int q = 0; q < P; ++q) {
    float A[3][3], AT[3][3], Cm[3][3], CA[3][3], TCT[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        A[r][c] = T[(size_t)q * 9 + r * 3 + c];
        AT[r][c] = T[(size_t)q * 9 + c * 3 + r];
        Cm[r][c] = C0[(size_t)q * 9 + r * 3 + c];
      }
    matmul3(Cm, A, CA);
    matmul3(AT, CA, TCT);
    const float* m = imp0 + (size_t)q * 3;
    for (int r = 0; r < 3; ++r)
      for (int a = 0; a < 3; ++a) {
        float gm = 0.f;
        if (gT) {
          const float* G = gT + (size_t)q * 27 + r * 9 + a * 3;
          gm = G[0] * m[0] + G[1] * m[1] + G[2] * m[2];
        }
        C[(size_t)q * 9 + r * 3 + a] = gm + TCT[r][a];
      }
  }
}

// compute_dT_dx: 3D/run_3D.py:353-390, with the cell lists of get_particles_id_in_every_cell
// (3D/run_3D.py:342-351) built from pos in index order and capped at cap; neighbour cells
// outside the grid are skipped.  pos, pos0 [P][3]; T [P][3][3]; gT [P][3][3][3].
void oracle3_compute_dT_dx(const float* pos, const float* pos0, const float* T, int P, int nx, int ny, int nz,
                           double dx, int cap, float* gT) {
  const float dxr = float(dx);
  const float inv = float(1.0 / dx);
  const size_t C = (size_t)nx * ny * nz;
  std::vector<std::vector<int>> lists(C);
  for (int q = 0; q < P; ++q) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
      int v = (int)(pos[(size_t)q * 3 + a] / dxr);
      c[a] = clampi(v, 0, (a == 0 ? nx : (a == 1 ? ny : nz)) - 1);
    }
    std::vector<int>& L = lists[((size_t)c[0] * ny + c[1]) * nz + c[2]];
    if ((int)L.size() < cap) L.push_back(q);
  }
#pragma omp parallel for schedule(static)
  for (int q = 0; q < P; ++q) {
    float acc[3][3][3] = {{{0}}};
    const float* xi = pos0 + (size_t)q * 3;
    int base[3] = {(int)(xi[0] / dxr), (int)(xi[1] / dxr), (int)(xi[2] / dxr)};
    for (int oi = -1; oi < 3; ++oi)
      for (int oj = -1; oj < 3; ++oj)
        for (int ok = -1; ok < 3; ++ok) {
          int ci = base[0] + oi, cj = base[1] + oj, ck = base[2] + ok;
          if (ci < 0 || ci >= nx || cj < 0 || cj >= ny || ck < 0 || ck >= nz) continue;
          for (int n : lists[((size_t)ci * ny + cj) * nz + ck]) {
            const float* xn = pos0 + (size_t)n * 3;
            float d0 = xn[0] - xi[0], d1 = xn[1] - xi[1], d2 = xn[2] - xi[2];
            float dw[3] = {inv * dN2(d0) * N2(d1) * N2(d2), inv * N2(d0) * dN2(d1) * N2(d2),
                           inv * N2(d0) * N2(d1) * dN2(d2)};
            const float* Tn = T + (size_t)n * 9;
            for (int r = 0; r < 3; ++r)
              for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) acc[r][a][b] += dw[a] * Tn[b * 3 + r];
          }
        }
    for (int r = 0; r < 3; ++r)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) gT[(size_t)q * 27 + r * 9 + a * 3 + b] = acc[r][a][b];
  }
}

}  // extern "C"
