/*
 * associative_cta.cuh -- the associative-scan smoother for larger state
 * dimensions, one thread block (CTA) per element or combine.  Included by
 * associative.cu (it uses that file's find_track and ScanLevel).
 *
 * Same algorithm and arithmetic as the per-thread kernels of associative.cu
 * (c/kalman_associative_smoother.c): filtering elements
 * (build_filtering_element_new 309-505), filtering and smoothing combines
 * (filteringAssociativeOperation 889-980, smoothingAssociativeOperation
 * 982-1016), smoothing elements (build_smoothing_element_new 697-753) and the
 * read-outs (1054-1091).  Every n x n product runs with one thread per output
 * entry and every solve as a Householder QR of [A | B] with one thread per
 * column (cta_linalg.cuh), on row-major matrices in a per-CTA region of global
 * scratch; grids are persistent.  Element arrays are slot-major (all entries
 * of an element contiguous).  FP64.
 */
#pragma once
#include "cta_linalg.cuh"

namespace acta {

using ::cta::Aos;
using ::cta::NT;

/* filtering elements (A, b, Z, e, J) and smoothing elements (E, g, L):
 * matrices column-major inside an element, (p, q) at entry q * n + p */
struct FEl {
  Aos<double> A, Z, J, b, e;
};
struct SEl {
  Aos<double> E, L, g;
};

struct AArgs {
  int n, ntracks;
  const int64_t* track_start;
  double* state;
  double* cov;
  int* flag;
  double* scratch;
  int64_t scratch_per_cta;
};

struct RawS {
  const double *F, *c, *K, *G, *o, *C;
  const char *K_type, *C_type;
  const int32_t* obs_rows;
  int mmax;
};

/* row-major matrix in scratch */
struct M {
  double* p;
  int ld;
  __device__ __forceinline__ double& operator()(int r, int c) const { return p[(int64_t)r * ld + c]; }
};

/* out(i, j) = (acc ? out(i, j) : 0) + alpha sum_l a(i, l) b(l, j), i < r, j < c;
 * one thread per output entry (consecutive threads: consecutive j) */
template <class FA, class FB, class FO>
__device__ __forceinline__ void gemm(int r, int c, int k, FA a, FB b, FO out, double alpha, bool acc)
{
  for (int e = threadIdx.x; e < r * c; e += NT) {
    const int i = e / c, j = e - i * c;
    double s = 0.0;
    for (int l = 0; l < k; ++l) s = fma(a(i, l), b(l, j), s);
    out(i, j) = acc ? fma(alpha, s, out(i, j)) : alpha * s;
  }
  __syncthreads();
}

/* W = [A | B] (n x (n+p), row-major, ld n+p): W[:, n:n+p] <- A^{-1} B by
 * Householder QR and back-substitution; true (every thread) on a zero pivot */
__device__ bool solve_square(M W, int n, int p, double* red)
{
  ::cta::householder(W.p, W.ld, n, n, n + p, red);
  __shared__ int zero;
  if (threadIdx.x == 0) {
    zero = 0;
    for (int i = 0; i < n; ++i)
      if (W(i, i) == 0.0) zero = 1;
  }
  __syncthreads();
  const bool bad = zero != 0;
  if (!bad) ::cta::solve_upper_cols(W.p, W.ld, n, W.p, W.ld, n, n + p);
  __syncthreads();
  return bad;
}

/* the explicit covariance of a factor (kalman_covariance_matrix_explicit,
 * c/kalman_base.c:178-214) into out (dim x dim); ws: dim x 2 dim */
__device__ bool explicit_cov(char type, const double* cov, int ldc, int dim, M out, M ws, double* red)
{
  const int tid = threadIdx.x;
  if (type == 'C') {
    for (int e = tid; e < dim * dim; e += NT) out(e / dim, e % dim) = cov[(int64_t)(e % dim) * ldc + e / dim];
    __syncthreads();
    return false;
  }
  if (type == 'w') {
    for (int e = tid; e < dim * dim; e += NT) {
      const int i = e / dim, j = e % dim;
      out(i, j) = i == j ? 1.0 / (cov[i] * cov[i]) : 0.0;
    }
    __syncthreads();
    return false;
  }
  if (type == 'U' || type == 'F') { /* L L^T */
    gemm(dim, dim, dim, [&](int i, int l) { return l <= i ? cov[(int64_t)l * ldc + i] : 0.0; },
         [&](int l, int j) { return l <= j ? cov[(int64_t)l * ldc + j] : 0.0; }, [&](int i, int j) -> double& { return out(i, j); },
         1.0, false);
    return false;
  }
  if (type == 'W') { /* (W^T W)^{-1} = W^{-1} W^{-T} */
    for (int e = tid; e < dim * 2 * dim; e += NT) {
      const int i = e / (2 * dim), j = e % (2 * dim);
      ws(i, j) = j < dim ? cov[(int64_t)j * ldc + i] : (j - dim == i ? 1.0 : 0.0);
    }
    __syncthreads();
    const bool bad = solve_square(ws, dim, dim, red);
    gemm(dim, dim, dim, [&](int i, int l) { return ws(i, dim + l); }, [&](int l, int j) { return ws(j, dim + l); },
         [&](int i, int j) -> double& { return out(i, j); }, 1.0, false);
    return bad;
  }
  return true;
}

/* filtering elements, one CTA per step (persistent); step i of a track writes
 * element r = i - 1 of its sequence, step 0 writes its filtered estimate. */
__global__ void __launch_bounds__(NT) element_cta(AArgs a, RawS raw, FEl out, const int64_t* seq_start,
                                                  int64_t nsteps)
{
  __shared__ double red[33];
  const int n = a.n, mm = raw.mmax, tid = threadIdx.x;
  const int64_t nn = (int64_t)n * n;
  const int mxr = n > mm ? n : mm;
  double* base = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  /* scratch: m0 (n) | P0 (nn) | Kx (nn) | T (mxr x 2n) | WS (mxr x (mxr+n+1)) | L (mxr^2) | S (mxr^2) |
     GtS (n x mxr) | Kg (n x mxr) | v (2 mxr) | tmp (mxr x NT) */
  double* m0 = base;
  const M P0{m0 + n, n}, Kx{P0.p + nn, n}, T{Kx.p + nn, 2 * n};
  const M WS{T.p + (int64_t)mxr * 2 * n, mxr + n + 1};
  const M Lm{WS.p + (int64_t)mxr * (mxr + n + 1), mxr}, S{Lm.p + (int64_t)mxr * mxr, mxr};
  const M GtS{S.p + (int64_t)mxr * mxr, mxr}, Kg{GtS.p + (int64_t)n * mxr, mxr};
  double* v = Kg.p + (int64_t)n * mxr;
  double* tmp = v + 2 * mxr;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t g0 = a.track_start[t], i = g - g0;
    bool bad = false;
    if (i <= 1) { /* m0 = R^{-1} Q^T (W o_0), P0 = R^{-1} R^{-T} from the square step-0 observation */
      const int m = raw.obs_rows[g0];
      if (m != n) {
        if (tid == 0) atomicOr(a.flag, 4);
        __syncthreads();
        continue;
      }
      const char ct = raw.C_type[g0];
      if (tid == 0 && !::cta::valid_cov_type(ct)) atomicOr(a.flag, 4);
      const M W{WS.p, n + 1};
      for (int e = tid; e < n * (n + 1); e += NT) {
        const int r = e / (n + 1), c = e - r * (n + 1);
        W(r, c) = c < n ? raw.G[g0 * (int64_t)mm * n + (int64_t)c * mm + r] : raw.o[g0 * mm + r];
      }
      __syncthreads();
      bad |= !::cta::weigh_panel(ct, raw.C + g0 * (int64_t)mm * mm, mm, n, W.p, W.ld, n + 1, Lm.p, red, tmp);
      ::cta::householder(W.p, W.ld, n, n, n + 1, red);
      if (tid == 0)
        for (int r = 0; r < n; ++r)
          if (W(r, r) == 0.0) bad = true;
      for (int r = tid; r < n; r += NT) m0[r] = W(r, n);
      __syncthreads();
      ::cta::solve_upper_vec(W.p, W.ld, n, m0);
      /* Ri = R^{-1} into T (n x n, ld 2n), P0 = Ri Ri^T */
      for (int e = tid; e < n * n; e += NT) T(e / n, e % n) = (e / n == e % n) ? 1.0 : 0.0;
      __syncthreads();
      ::cta::solve_upper_cols(W.p, W.ld, n, T.p, T.ld, 0, n);
      gemm(n, n, n, [&](int r, int l) { return T(r, l); }, [&](int l, int c) { return T(c, l); },
           [&](int r, int c) -> double& { return P0(r, c); }, 1.0, false);
      if (i == 0) {
        for (int r = tid; r < n; r += NT) a.state[g0 * n + r] = m0[r];
        for (int e = tid; e < n * n; e += NT) a.cov[g0 * nn + e] = P0(e % n, e / n);
        if (bad && tid == 0) atomicOr(a.flag, 2);
        __syncthreads();
        continue;
      }
    }
    const int64_t r = seq_start[t] + (i - 1);
    const double* F = raw.F + g * nn; /* F(p, q) at F[q * n + p] */
    const double* c = raw.c + g * n;
    auto Fm = [&](int p, int q) { return F[(int64_t)q * n + p]; };
    const char kt = raw.K_type[g];
    if (tid == 0 && !::cta::valid_cov_type(kt)) atomicOr(a.flag, 4);
    bad |= explicit_cov(kt, raw.K + g * nn, n, n, Kx, M{WS.p, 2 * n}, red);
    if (i == 1) { /* Kx += F P0 F^T */
      gemm(n, n, n, Fm, [&](int l, int q) { return P0(l, q); }, [&](int p, int q) -> double& { return T(p, q); }, 1.0,
           false);
      gemm(n, n, n, [&](int p, int l) { return T(p, l); }, [&](int l, int q) { return Fm(q, l); },
           [&](int p, int q) -> double& { return Kx(p, q); }, 1.0, true);
    }
    int m = raw.obs_rows[g];
    if (m < 0 || m > mm) {
      m = 0;
      if (tid == 0) atomicOr(a.flag, 4);
    }
    if (m == 0) {
      for (int e = tid; e < n * n; e += NT) {
        const int p = e % n, q = e / n;
        out.Z.at(e, r) = Kx(p, q);
        out.A.at(e, r) = i == 1 ? 0.0 : Fm(p, q);
        out.J.at(e, r) = 0.0;
      }
      for (int p = tid; p < n; p += NT) {
        double bp = c[p];
        if (i == 1)
          for (int k = 0; k < n; ++k) bp = fma(Fm(p, k), m0[k], bp);
        out.b.at(p, r) = bp;
        out.e.at(p, r) = 0.0;
      }
      if (bad && tid == 0) atomicOr(a.flag, 2);
      __syncthreads();
      continue;
    }
    const double* G = raw.G + g * (int64_t)mm * n;
    auto Gm = [&](int p, int q) { return G[(int64_t)q * mm + p]; };
    const double* o = raw.o + g * mm;
    const char ct = raw.C_type[g];
    if (tid == 0 && !::cta::valid_cov_type(ct)) atomicOr(a.flag, 4);
    bad |= explicit_cov(ct, raw.C + g * (int64_t)mm * mm, mm, m, S, M{WS.p, 2 * m}, red); /* S = C */
    /* S += G Kx G^T: T = G Kx (m x n), then S += T G^T */
    gemm(m, n, n, Gm, [&](int l, int q) { return Kx(l, q); }, [&](int p, int q) -> double& { return T(p, q); }, 1.0,
         false);
    gemm(m, m, n, [&](int p, int l) { return T(p, l); }, [&](int l, int q) { return Gm(q, l); },
         [&](int p, int q) -> double& { return S(p, q); }, 1.0, true);
    /* W = [S^T | G] (m x (m+n)): X = S^{-T} G, GtS = X^T (n x m) */
    {
      const M W{WS.p, m + n};
      for (int e = tid; e < m * (m + n); e += NT) {
        const int p = e / (m + n), q = e - p * (m + n);
        W(p, q) = q < m ? S(q, p) : Gm(p, q - m);
      }
      __syncthreads();
      bad |= solve_square(W, m, n, red);
      for (int e = tid; e < n * m; e += NT) {
        const int p = e / m, q = e - p * m;
        GtS(p, q) = W(q, m + p);
      }
      __syncthreads();
    }
    /* Kg = Kx GtS (n x m); res = o - G c into v[0:m] */
    gemm(n, m, n, [&](int p, int l) { return Kx(p, l); }, [&](int l, int q) { return GtS(l, q); },
         [&](int p, int q) -> double& { return Kg(p, q); }, 1.0, false);
    for (int p = tid; p < m; p += NT) {
      double s = o[p];
      for (int k = 0; k < n; ++k) s = fma(-Gm(p, k), c[k], s);
      v[p] = s;
    }
    __syncthreads();
    if (i == 1) {
      /* m1 = F m0 + c into tmp[0:n]; b = m1 + Kg (o - G m1); Z = Kx - Kg S Kg^T; A = 0 */
      double* m1 = tmp;
      double* d = tmp + n;
      for (int p = tid; p < n; p += NT) {
        double s = c[p];
        for (int k = 0; k < n; ++k) s = fma(Fm(p, k), m0[k], s);
        m1[p] = s;
      }
      __syncthreads();
      for (int p = tid; p < m; p += NT) {
        double s = o[p];
        for (int k = 0; k < n; ++k) s = fma(-Gm(p, k), m1[k], s);
        d[p] = s;
      }
      __syncthreads();
      for (int p = tid; p < n; p += NT) {
        double s = m1[p];
        for (int k = 0; k < m; ++k) s = fma(Kg(p, k), d[k], s);
        out.b.at(p, r) = s;
      }
      /* T = Kg S (n x m) */
      gemm(n, m, m, [&](int p, int l) { return Kg(p, l); }, [&](int l, int q) { return S(l, q); },
           [&](int p, int q) -> double& { return T(p, q); }, 1.0, false);
      for (int e = tid; e < n * n; e += NT) {
        const int p = e % n, q = e / n;
        double s = Kx(p, q);
        for (int k = 0; k < m; ++k) s = fma(-T(p, k), Kg(q, k), s);
        out.Z.at(e, r) = s;
        out.A.at(e, r) = 0.0;
      }
      __syncthreads();
    } else {
      /* b = c + Kg res; T[:, 0:n] = G F (m x n), T[:, n:2n] = G Kx; A = F - Kg (G F), Z = Kx - Kg (G Kx) */
      for (int p = tid; p < n; p += NT) {
        double s = c[p];
        for (int k = 0; k < m; ++k) s = fma(Kg(p, k), v[k], s);
        out.b.at(p, r) = s;
      }
      gemm(m, 2 * n, n, Gm, [&](int l, int q) { return q < n ? Fm(l, q) : Kx(l, q - n); },
           [&](int p, int q) -> double& { return T(p, q); }, 1.0, false);
      for (int e = tid; e < n * n; e += NT) {
        const int p = e % n, q = e / n;
        double sa = Fm(p, q), sz = Kx(p, q);
        for (int k = 0; k < m; ++k) {
          sa = fma(-Kg(p, k), T(k, q), sa);
          sz = fma(-Kg(p, k), T(k, n + q), sz);
        }
        out.A.at(e, r) = sa;
        out.Z.at(e, r) = sz;
      }
      __syncthreads();
    }
    /* e = F^T (GtS res); J = F^T GtS (G F) */
    double* u = tmp; /* GtS res (n) */
    for (int p = tid; p < n; p += NT) {
      double s = 0.0;
      for (int k = 0; k < m; ++k) s = fma(GtS(p, k), v[k], s);
      u[p] = s;
    }
    __syncthreads();
    for (int p = tid; p < n; p += NT) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(Fm(k, p), u[k], s);
      out.e.at(p, r) = s;
    }
    /* T = G F (m x n), U = GtS T (n x n, in L's storage), J = F^T U */
    gemm(m, n, n, Gm, [&](int l, int q) { return Fm(l, q); }, [&](int p, int q) -> double& { return T(p, q); }, 1.0,
         false);
    const M U{Lm.p, n};
    gemm(n, n, m, [&](int p, int l) { return GtS(p, l); }, [&](int l, int q) { return T(l, q); },
         [&](int p, int q) -> double& { return U(p, q); }, 1.0, false);
    for (int e = tid; e < n * n; e += NT) {
      const int p = e % n, q = e / n;
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = fma(Fm(k, p), U(k, q), s);
      out.J.at(e, r) = s;
    }
    if (bad && tid == 0) atomicOr(a.flag, 2);
    __syncthreads();
  }
}

/* the filtering combine O = Xi (x) Xj; O may alias Xj (every entry of Xj is
 * read before O's entry at the same place is written).  Scratch: W
 * (n x 2n) | Xm | Ym | T (n x n each) | the outputs (2 n^2 + 4 n). */
__device__ bool combine_filter(int n, const FEl& Xi, int64_t i, const FEl& Xj, int64_t j, const FEl& O, int64_t o,
                               double* ws, double* red)
{
  const int tid = threadIdx.x;
  const M W{ws, 2 * n}, Xm{ws + 2 * (int64_t)n * n, n}, Ym{Xm.p + (int64_t)n * n, n}, T{Ym.p + (int64_t)n * n, n};
  double* extra = T.p + (int64_t)n * n;
  auto A_i = [&](int p, int q) { return Xi.A.at(q * n + p, i); };
  auto Z_i = [&](int p, int q) { return Xi.Z.at(q * n + p, i); };
  auto J_i = [&](int p, int q) { return Xi.J.at(q * n + p, i); };
  auto A_j = [&](int p, int q) { return Xj.A.at(q * n + p, j); };
  auto Z_j = [&](int p, int q) { return Xj.Z.at(q * n + p, j); };
  auto J_j = [&](int p, int q) { return Xj.J.at(q * n + p, j); };
  bool bad = false;
  /* X = Aj (I + Zi Jj)^{-1}: solve (I + Zi Jj)^T X^T = Aj^T */
  gemm(n, n, n, [&](int p, int l) { return J_j(l, p); }, [&](int l, int q) { return Z_i(q, l); },
       [&](int p, int q) -> double& { return W(p, q); }, 1.0, false); /* (Zi Jj)^T */
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    if (p == q) W(p, q) += 1.0;
    W(p, n + q) = A_j(q, p);
  }
  __syncthreads();
  bad |= solve_square(W, n, n, red);
  for (int e = tid; e < n * n; e += NT) Xm(e / n, e % n) = W(e % n, n + e / n);
  __syncthreads();
  /* Y = Ai^T (I + Jj Zi)^{-1}: solve (I + Jj Zi)^T Y^T = Ai */
  gemm(n, n, n, [&](int p, int l) { return Z_i(l, p); }, [&](int l, int q) { return J_j(q, l); },
       [&](int p, int q) -> double& { return W(p, q); }, 1.0, false); /* (Jj Zi)^T */
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    if (p == q) W(p, q) += 1.0;
    W(p, n + q) = A_i(p, q);
  }
  __syncthreads();
  bad |= solve_square(W, n, n, red);
  for (int e = tid; e < n * n; e += NT) Ym(e / n, e % n) = W(e % n, n + e / n);
  __syncthreads();
  /* b = X (bi + Zi ej) + bj, e = Y (ej - Jj bi) + ei: vectors in W's first row block */
  double* v1 = extra;
  double* v2 = extra + n;
  for (int p = tid; p < n; p += NT) {
    double s1 = Xi.b.at(p, i), s2 = Xj.e.at(p, j);
    for (int k = 0; k < n; ++k) {
      s1 = fma(Z_i(p, k), Xj.e.at(k, j), s1);
      s2 = fma(-J_j(p, k), Xi.b.at(k, i), s2);
    }
    v1[p] = s1;
    v2[p] = s2;
  }
  __syncthreads();
  /* T = X Zi, then Z = T Aj^T + Zj (into W's n x n block at ld 2n, cols 0..n) */
  gemm(n, n, n, [&](int p, int l) { return Xm(p, l); }, Z_i, [&](int p, int q) -> double& { return T(p, q); }, 1.0,
       false);
  double* Zo = extra + 2 * n; /* n x n at ld n, after v1, v2 */
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    double s = Z_j(p, q);
    for (int k = 0; k < n; ++k) s = fma(T(p, k), A_j(q, k), s);
    Zo[e] = s;
  }
  double* bo = Zo + (int64_t)n * n;
  double* eo = bo + n;
  for (int p = tid; p < n; p += NT) {
    double sb = Xj.b.at(p, j), se = Xi.e.at(p, i);
    for (int k = 0; k < n; ++k) {
      sb = fma(Xm(p, k), v1[k], sb);
      se = fma(Ym(p, k), v2[k], se);
    }
    bo[p] = sb;
    eo[p] = se;
  }
  __syncthreads();
  /* J = Y (Jj Ai) + Ji: T = Jj Ai */
  gemm(n, n, n, J_j, A_i, [&](int p, int q) -> double& { return T(p, q); }, 1.0, false);
  double* Jo = eo + n;
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    double s = J_i(p, q);
    for (int k = 0; k < n; ++k) s = fma(Ym(p, k), T(k, q), s);
    Jo[e] = s;
  }
  __syncthreads();
  /* A = X Ai into T, then write every output (Xj may be O) */
  gemm(n, n, n, [&](int p, int l) { return Xm(p, l); }, A_i, [&](int p, int q) -> double& { return T(p, q); }, 1.0,
       false);
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    O.Z.at(q * n + p, o) = Zo[e];
    O.J.at(q * n + p, o) = Jo[e];
    O.A.at(q * n + p, o) = T(p, q);
  }
  for (int p = tid; p < n; p += NT) {
    O.b.at(p, o) = bo[p];
    O.e.at(p, o) = eo[p];
  }
  __syncthreads();
  return bad;
}

/* the smoothing combine: E = Ej Ei, g = Ej gi + gj, L = Ej Li Ej^T + Lj */
__device__ bool combine_smooth(int n, const SEl& Xi, int64_t i, const SEl& Xj, int64_t j, const SEl& O, int64_t o,
                               double* ws, double*)
{
  const int tid = threadIdx.x;
  const M T{ws, n}, U{ws + (int64_t)n * n, n}, Lo{U.p + (int64_t)n * n, n};
  double* go = Lo.p + (int64_t)n * n;
  auto E_j = [&](int p, int q) { return Xj.E.at(q * n + p, j); };
  gemm(n, n, n, E_j, [&](int l, int q) { return Xi.L.at(q * n + l, i); }, [&](int p, int q) -> double& { return T(p, q); },
       1.0, false);
  gemm(n, n, n, E_j, [&](int l, int q) { return Xi.E.at(q * n + l, i); }, [&](int p, int q) -> double& { return U(p, q); },
       1.0, false);
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    double s = Xj.L.at(q * n + p, j);
    for (int k = 0; k < n; ++k) s = fma(T(p, k), E_j(q, k), s);
    Lo(p, q) = s;
  }
  for (int p = tid; p < n; p += NT) {
    double s = Xj.g.at(p, j);
    for (int k = 0; k < n; ++k) s = fma(E_j(p, k), Xi.g.at(k, i), s);
    go[p] = s;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += NT) {
    const int p = e / n, q = e - p * n;
    O.L.at(q * n + p, o) = Lo(p, q);
    O.E.at(q * n + p, o) = U(p, q);
  }
  for (int p = tid; p < n; p += NT) O.g.at(p, o) = go[p];
  __syncthreads();
  return false;
}

__device__ void copy_elem(int n, const FEl& X, int64_t i, const FEl& O, int64_t o)
{
  for (int e = threadIdx.x; e < n * n; e += NT) {
    O.A.at(e, o) = X.A.at(e, i);
    O.Z.at(e, o) = X.Z.at(e, i);
    O.J.at(e, o) = X.J.at(e, i);
  }
  for (int e = threadIdx.x; e < n; e += NT) {
    O.b.at(e, o) = X.b.at(e, i);
    O.e.at(e, o) = X.e.at(e, i);
  }
  __syncthreads();
}
__device__ void copy_elem(int n, const SEl& X, int64_t i, const SEl& O, int64_t o)
{
  for (int e = threadIdx.x; e < n * n; e += NT) {
    O.E.at(e, o) = X.E.at(e, i);
    O.L.at(e, o) = X.L.at(e, i);
  }
  for (int e = threadIdx.x; e < n; e += NT) O.g.at(e, o) = X.g.at(e, i);
  __syncthreads();
}

__device__ __forceinline__ bool combine(int n, const FEl& Xi, int64_t i, const FEl& Xj, int64_t j, const FEl& O,
                                        int64_t o, double* ws, double* red)
{
  return combine_filter(n, Xi, i, Xj, j, O, o, ws, red);
}
__device__ __forceinline__ bool combine(int n, const SEl& Xi, int64_t i, const SEl& Xj, int64_t j, const SEl& O,
                                        int64_t o, double* ws, double* red)
{
  return combine_smooth(n, Xi, i, Xj, j, O, o, ws, red);
}

template <class El>
__global__ void __launch_bounds__(NT) up_cta(int n, int T, ScanLevel lv, ScanLevel nx, El cur, El nxt, int* flag,
                                             double* scratch, int64_t per_cta)
{
  __shared__ double red[33];
  double* ws = scratch + (int64_t)blockIdx.x * per_cta;
  for (int64_t item = blockIdx.x; item < lv.nup; item += gridDim.x) {
    const int t = find_track(lv.up_items, T, item);
    const int64_t p = item - lv.up_items[t];
    const int64_t s0 = lv.start[t] + 2 * p, o = nx.start[t] + p;
    if (2 * p + 1 < lv.L[t]) {
      if (combine(n, cur, s0, cur, s0 + 1, nxt, o, ws, red) && threadIdx.x == 0) atomicOr(flag, 2);
    } else {
      copy_elem(n, cur, s0, nxt, o);
    }
  }
}

template <class El>
__global__ void __launch_bounds__(NT) down_cta(int n, int T, ScanLevel lv, ScanLevel nx, El cur, El nxt, int* flag,
                                               double* scratch, int64_t per_cta)
{
  __shared__ double red[33];
  double* ws = scratch + (int64_t)blockIdx.x * per_cta;
  for (int64_t item = blockIdx.x; item < lv.ndown; item += gridDim.x) {
    const int t = find_track(lv.down_items, T, item);
    const int64_t p = item - lv.down_items[t];
    const int64_t L = lv.L[t];
    if (L < 2) continue;
    const int64_t s0 = lv.start[t] + 2 * p, b0 = nx.start[t] + p;
    if (2 * p + 1 < L) copy_elem(n, nxt, b0, cur, s0 + 1);
    if (p > 0 && combine(n, nxt, b0 - 1, cur, s0, cur, s0, ws, red) && threadIdx.x == 0) atomicOr(flag, 2);
  }
}

/* filtered estimates: step i >= 1 of each track gets (b, Z) of prefix i-1 */
__global__ void filtered_out_cta(AArgs a, FEl el, const int64_t* seq_start, int64_t nsteps)
{
  const int n = a.n;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t i = g - a.track_start[t];
    if (i == 0) continue;
    const int64_t r = seq_start[t] + i - 1;
    for (int p = threadIdx.x; p < n; p += blockDim.x) a.state[g * n + p] = el.b.at(p, r);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) a.cov[g * (int64_t)n * n + e] = el.Z.at(e, r);
  }
}

/* smoothing elements, reversed: step i of a track of length k is element
 * r = k-1-i.  E = P F^T (F P F^T + Q)^{-1}, g = x - E (F x + c), L = P - E F P */
__global__ void __launch_bounds__(NT) smooth_element_cta(AArgs a, RawS raw, SEl out, const int64_t* seq_start,
                                                         int64_t nsteps)
{
  __shared__ double red[33];
  const int n = a.n, tid = threadIdx.x;
  const int64_t nn = (int64_t)n * n;
  double* base = a.scratch + (int64_t)blockIdx.x * a.scratch_per_cta;
  const M Q{base, n}, PFt{base + nn, n}, W{base + 2 * nn, 2 * n}, Em{base + 4 * nn, n}, CW{base + 5 * nn, 2 * n};
  double* v = base + 7 * nn;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t g0 = a.track_start[t], k = a.track_start[t + 1] - g0, i = g - g0;
    const int64_t r = seq_start[t] + (k - 1 - i);
    const double* x = a.state + g * n;
    const double* P = a.cov + g * nn; /* P(p, q) at P[q * n + p] */
    if (i == k - 1) {
      for (int e = tid; e < n * n; e += NT) {
        out.E.at(e, r) = 0.0;
        out.L.at(e, r) = P[e];
      }
      for (int p = tid; p < n; p += NT) out.g.at(p, r) = x[p];
      __syncthreads();
      continue;
    }
    const int64_t g1 = g + 1;
    const double* F = raw.F + g1 * nn;
    const double* c = raw.c + g1 * n;
    auto Fm = [&](int p, int q) { return F[(int64_t)q * n + p]; };
    auto Pm = [&](int p, int q) { return P[(int64_t)q * n + p]; };
    bool bad = explicit_cov(raw.K_type[g1], raw.K + g1 * nn, n, n, Q, CW, red);
    /* PFt = P F^T */
    gemm(n, n, n, Pm, [&](int l, int q) { return Fm(q, l); }, [&](int p, int q) -> double& { return PFt(p, q); }, 1.0,
         false);
    /* W = [(F P F^T + Q)^T | (P F^T)^T]; the solve gives E^T */
    gemm(n, n, n, Fm, [&](int l, int q) { return PFt(l, q); }, [&](int p, int q) -> double& { return W(q, p); }, 1.0,
         false); /* W(q, p) = (F P F^T)(p, q) */
    for (int e = tid; e < n * n; e += NT) {
      const int p = e / n, q = e - p * n;
      W(p, q) += Q(q, p);
      W(p, n + q) = PFt(q, p);
    }
    __syncthreads();
    bad |= solve_square(W, n, n, red);
    for (int e = tid; e < n * n; e += NT) Em(e / n, e % n) = W(e % n, n + e / n);
    __syncthreads();
    /* g = x - E (F x + c) */
    for (int p = tid; p < n; p += NT) {
      double s = c[p];
      for (int l = 0; l < n; ++l) s = fma(Fm(p, l), x[l], s);
      v[p] = s;
    }
    __syncthreads();
    for (int p = tid; p < n; p += NT) {
      double s = x[p];
      for (int l = 0; l < n; ++l) s = fma(-Em(p, l), v[l], s);
      out.g.at(p, r) = s;
    }
    /* L = P - (E F) P: EF into Q */
    gemm(n, n, n, [&](int p, int l) { return Em(p, l); }, Fm, [&](int p, int q) -> double& { return Q(p, q); }, 1.0,
         false);
    for (int e = tid; e < n * n; e += NT) {
      const int p = e % n, q = e / n;
      double s = Pm(p, q);
      for (int l = 0; l < n; ++l) s = fma(-Q(p, l), Pm(l, q), s);
      out.L.at(e, r) = s;
      out.E.at(e, r) = Em(p, q);
    }
    if (bad && tid == 0) atomicOr(a.flag, 2);
    __syncthreads();
  }
}

__global__ void smoothed_out_cta(AArgs a, SEl el, const int64_t* seq_start, int64_t nsteps)
{
  const int n = a.n;
  for (int64_t g = blockIdx.x; g < nsteps; g += gridDim.x) {
    const int t = find_track(a.track_start, a.ntracks, g);
    const int64_t g0 = a.track_start[t], k = a.track_start[t + 1] - g0, i = g - g0;
    const int64_t r = seq_start[t] + (k - 1 - i);
    for (int p = threadIdx.x; p < n; p += blockDim.x) a.state[g * n + p] = el.g.at(p, r);
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) a.cov[g * (int64_t)n * n + e] = el.L.at(e, r);
  }
}

}  // namespace acta
