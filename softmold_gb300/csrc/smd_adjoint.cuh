// Adjoint of the Langevin velocity-Verlet step (no reference counterpart: the
// reference has no derivatives).  One loop iteration of MD.cpp:335-729 with
// the box fixed maps the state (x_n, h_n), h the half-step velocity, to
//   h_{n+1} = (1 - gamma dt) h_n + dt F(x_n; theta) + dt sigma psi_n
//   x_{n+1} = x_n + dt h_{n+1}
// (verlet.h:288-355, 463-491 and langevin.h:284-331 composed), and the
// observable is J = (1/T) sum_{n=1..T} U(x_n; theta).  With the Langevin
// noise fixed by its seed, the discrete adjoint runs backwards as
//   w_n    = hbar_{n+1} + dt xbar_{n+1}
//   xbar_n = xbar_{n+1} + dt K(x_n) w_n - (1/T) F(x_n)
//   hbar_n = (1 - gamma dt) w_n
//   dJ/dtheta = sum_n [ dt w_n . dF(x_n)/dtheta + (1/T) dU(x_n)/dtheta ]
// where K = dF/dx is the symmetric force Jacobian (minus the Hessian of U).
// K w is a Hessian-vector product over the same Verlet list as the forces:
// for a pair force g(r) d, d = x_i - x_j,
//   (K w)_i = sum_j g (w_i - w_j) + (g'(r)/r) (d . (w_i - w_j)) d.
// The parameters enter linearly: Umin of a type pair through the table rows
// (include/potentials/laradjiRevalee.h:84-152), kbond and kbend as the CHAIN
// constants 1 and 3 (include/MD.h:384-431, 683-789), so their derivatives
// are the same kernels evaluated with derivative rows or unit constants.
//
// MIXED: pair terms in FP32 from the exact fractional mirror, every sum and
// the adjoint state in FP64.  PLAIN: FP64 throughout.  The CHAIN terms are
// FP64 in both, their K w from forward-mode dual numbers through the force
// formulas.
#pragma once

#include "smd_kernels.cuh"

namespace smd {

// ------------------------------------------------------------ dual numbers
struct Dd {  // value and directional derivative
  double v, t;
};
__device__ __forceinline__ Dd operator+(Dd a, Dd b) { return {a.v + b.v, a.t + b.t}; }
__device__ __forceinline__ Dd operator-(Dd a, Dd b) { return {a.v - b.v, a.t - b.t}; }
__device__ __forceinline__ Dd operator-(Dd a) { return {-a.v, -a.t}; }
__device__ __forceinline__ Dd operator*(Dd a, Dd b) { return {a.v * b.v, a.t * b.v + a.v * b.t}; }
__device__ __forceinline__ Dd operator/(Dd a, Dd b) {
  const double q = a.v / b.v;
  return {q, (a.t - q * b.t) / b.v};
}
__device__ __forceinline__ Dd& operator+=(Dd& a, Dd b) { return a = a + b; }
__device__ __forceinline__ Dd& operator-=(Dd& a, Dd b) { return a = a - b; }
__device__ __forceinline__ Dd& operator/=(Dd& a, Dd b) { return a = a / b; }
__device__ __forceinline__ Dd sqrt(Dd a) {
  const double s = ::sqrt(a.v);
  return {s, a.t / (2.0 * s)};
}

// Device accumulators of one adjoint run.
struct AdjAcc {
  double J;         // (1/T) sum U
  double grad[3];   // dJ/d(Umin(a,b), kbond, kbend)
  double kw_norm;   // unused by the recursion; kept for diagnostics
};

// Derivative rows of the pair tables for Umin of one type pair (zero rows
// elsewhere), FP32 and FP64.
struct AdjTables {
  float fF[6 * kMaxTypes * kMaxTypes];
  float fU[6 * kMaxTypes * kMaxTypes];
  double dF[6 * kMaxTypes * kMaxTypes];
  double dU[6 * kMaxTypes * kMaxTypes];
};

// Positions of the state in file order (xs: 3n) written into the sorted
// arrays and the current mirror; the displacement from the list-build
// positions decides whether the list must be rebuilt before the next pass.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_adj_load(DevPtrs P, int cur, const double* xs, const double* vs) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  float vmax = 0.f;
  if (i < P.n) {
    const RepState& rs = P.rs[rep_of(P, i)];
    const int o = P.orig[i];
    const double x = xs[3 * o], y = xs[3 * o + 1], z = xs[3 * o + 2];
    P.x[i] = x;
    P.y[i] = y;
    P.z[i] = z;
    if (vs) {
      P.vx[i] = vs[3 * o];
      P.vy[i] = vs[3 * o + 1];
      P.vz[i] = vs[3 * o + 2];
    }
    const unsigned int fx = to_frac(x, rs.frac_per_len[0]), fy = to_frac(y, rs.frac_per_len[1]),
                       fz = to_frac(z, rs.frac_per_len[2]);
    vmax = displacement(P.ref[i], fx, fy, fz, rs);
    if constexpr (MIXED) {
      const uint4 me = P.m4[cur][i];
      P.m4[cur][i] = make_uint4(fx, fy, fz, me.w);
    } else {
      const double4 me = P.d4[cur][i];
      P.d4[cur][i] = make_double4(x, y, z, me.w);
    }
  }
  vmax = warp_max(vmax);
  __shared__ float smax[kBlock / 32];
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = vmax;
  __syncthreads();
  float bm = 0.f;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlock / 32; ++w) bm = fmaxf(bm, smax[w]);
  finalize_step(P, bm, StepEnd{0, 0, 0, 0, 0});
}

// Sorted-order copy of the adjoint direction w (file order) for the pair
// gathers.
template <typename V>
__global__ void __launch_bounds__(kBlock) k_adj_wsort(DevPtrs P, const double* w, V* ws) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const int o = P.orig[i];
  if constexpr (std::is_same<V, float4>::value)
    ws[i] = make_float4((float)w[3 * o], (float)w[3 * o + 1], (float)w[3 * o + 2], 0.f);
  else
    ws[i] = make_double4(w[3 * o], w[3 * o + 1], w[3 * o + 2], 0.0);
}

// Pair part of step n: for bead i the non-bonded force F_i, (K w)_i, and the
// replica sums of U, dU/dUmin and w_i . dF_i/dUmin.  G lanes per bead walk
// the Verlet list as k_force does; every sum is FP64.
template <bool MIXED, int G>
__global__ void __launch_bounds__(kBlock) k_adj_pair(DevPtrs P, int cur, const AdjTables* AT,
                                                     const typename std::conditional<MIXED, float4, double4>::type* ws,
                                                     double* kw, double* fpair, AdjAcc* acc, double dt, double invT) {
  using R = typename std::conditional<MIXED, float, double>::type;
  const Tables& T = *P.tab;
  const int t = blockIdx.x * kBlock + threadIdx.x;
  const int i = t / G, sub = t % G;
  const bool active = i < P.n;
  double F[3] = {0, 0, 0}, K[3] = {0, 0, 0}, u = 0, ut = 0, wft = 0;
  if (active) {
    const RepState& rs = P.rs[rep_of(P, i)];
    const int nn = P.nnbr[i];
    const int* nb = P.nbr + (size_t)i * P.kmax;
    const auto wi = ws[i];
    int ti;
    R mx, my, mz;
    uint4 mu = make_uint4(0, 0, 0, 0);
    if constexpr (MIXED) {
      mu = P.m4[cur][i];
      ti = mu.w & 0xff;
    } else {
      const double4 me = P.d4[cur][i];
      ti = __double_as_longlong(me.w) & 0xff;
      mx = me.x;
      my = me.y;
      mz = me.z;
    }
    const R* rowF;
    const R* rowU;
    const R* rowFt;
    const R* rowUt;
    if constexpr (MIXED) {
      rowF = T.fF + 6 * ti * T.nT;
      rowU = T.fU + 6 * ti * T.nT;
      rowFt = AT->fF + 6 * ti * T.nT;
      rowUt = AT->fU + 6 * ti * T.nT;
    } else {
      rowF = T.dF + 6 * ti * T.nT;
      rowU = T.dU + 6 * ti * T.nT;
      rowFt = AT->dF + 6 * ti * T.nT;
      rowUt = AT->dU + 6 * ti * T.nT;
    }
    const R rc2 = MIXED ? (R)T.rc2f : (R)T.rc2;
    for (int k = sub; k < nn; k += G) {
      const int j = __ldg(nb + k);
      R dx, dy, dz;
      int tj;
      if constexpr (MIXED) {
        const uint4 o = P.m4[cur][j];
        tj = o.w & 0xff;
        dx = frac_delta(mu.x, o.x, rs.len_per_frac[0]);
        dy = frac_delta(mu.y, o.y, rs.len_per_frac[1]);
        dz = frac_delta(mu.z, o.z, rs.len_per_frac[2]);
      } else {
        const double4 o = P.d4[cur][j];
        tj = __double_as_longlong(o.w) & 0xff;
        double ox = o.x, oy = o.y, oz = o.z;
        if (mx - ox > rs.box[0] / 2.0) ox += rs.box[0];
        if (mx - ox < -rs.box[0] / 2.0) ox -= rs.box[0];
        if (my - oy > rs.box[1] / 2.0) oy += rs.box[1];
        if (my - oy < -rs.box[1] / 2.0) oy -= rs.box[1];
        if (mz - oz > rs.box[2] / 2.0) oz += rs.box[2];
        if (mz - oz < -rs.box[2] / 2.0) oz -= rs.box[2];
        dx = mx - ox;
        dy = my - oy;
        dz = mz - oz;
      }
      const R r2 = dx * dx + dy * dy + dz * dz;
      if (!(r2 < rc2)) continue;
      const R rr = ::sqrt(r2);
      const R* c = rowF + 6 * tj;
      const int ci = (rr >= c[0]) ? 3 : 0;
      const R m = c[ci] - rr;
      const R g = ((c[ci + 1] - c[ci + 2] * m) * m) / rr;
      // g'(r)/r = -((C1 - 2 C2 m) + g) / r^2
      const R q = -((c[ci + 1] - (R)2 * c[ci + 2] * m) + g) / r2;
      const auto wj = ws[j];
      const R ex = (R)wi.x - (R)wj.x, ey = (R)wi.y - (R)wj.y, ez = (R)wi.z - (R)wj.z;
      const R dd = q * (dx * ex + dy * ey + dz * ez);
      F[0] += (double)(g * dx);
      F[1] += (double)(g * dy);
      F[2] += (double)(g * dz);
      K[0] += (double)(g * ex + dd * dx);
      K[1] += (double)(g * ey + dd * dy);
      K[2] += (double)(g * ez + dd * dz);
      u += 0.5 * (double)pair_pot<R>(rowU + 6 * tj, rr);
      const R* ct = rowFt + 6 * tj;
      if (ct[1] != (R)0 || ct[4] != (R)0) {
        const R mt = ct[ci] - rr;
        const R gt = ((ct[ci + 1] - ct[ci + 2] * mt) * mt) / rr;
        wft += (double)(gt * (dx * (R)wi.x + dy * (R)wi.y + dz * (R)wi.z));
        ut += 0.5 * (double)pair_pot<R>(rowUt + 6 * tj, rr);
      }
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    for (int d = 0; d < 3; ++d) {
      F[d] += __shfl_xor_sync(0xffffffffu, F[d], o);
      K[d] += __shfl_xor_sync(0xffffffffu, K[d], o);
    }
  }
  if (active && sub == 0) {
    for (int d = 0; d < 3; ++d) {
      kw[i + d * P.n] = K[d];
      fpair[i + d * P.n] = F[d];
    }
  }
  // replica sums (single-system handles): J and the Umin component
  const double gJ = invT * u, g0 = dt * wft + invT * ut;
  const double sJ = warp_sum(gJ), s0 = warp_sum(g0);
  if ((threadIdx.x & 31) == 0) {
    if (sJ != 0.0) atomicAdd(&acc->J, sJ);
    if (s0 != 0.0) atomicAdd(&acc->grad[0], s0);
  }
}

// CHAIN part of step n and the adjoint update of every bead (file order):
//   F_i = F_pair + F_chain, (K w)_i = (K w)_pair + (K w)_chain,
//   xbar += dt (K w)_i - invT F_i, hbar = (1 - gamma dt) w_i,
//   w_next = hbar + dt xbar.
// Adds invT U_chain and the kbond / kbend components to the accumulators.
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_adj_chain(DevPtrs P, int cur, const double* w, double* w_next,
                                                      double* xbar, double* hbar, const double* kw,
                                                      const double* fpair, AdjAcc* acc, double dt, double invT) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  double gJ = 0.0, g1 = 0.0, g2 = 0.0;
  if (i < P.n) {
    const Tables& T = *P.tab;
    const int r = rep_of(P, i);
    const RepParams& rp = P.rp[r];
    const RepState& rs = P.rs[r];
    const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
    const int o = P.orig[i];
    const double wi[3] = {w[3 * o], w[3 * o + 1], w[3 * o + 2]};
    double F[3] = {fpair[i], fpair[i + P.n], fpair[i + 2 * P.n]};
    double K[3] = {kw[i], kw[i + P.n], kw[i + 2 * P.n]};
    const int ci = P.cinfo[i];
    if (ci < 0 && !(ci & 0x40000000)) {
      const int p = ci & 0xfff, len = (ci >> 12) & 0xfff, set = (ci >> 24) & 0x1f;
      Vec3<double> e[4];
      bool valid[4];
      chain_vectors<MIXED, double>(P, cur, i, p, len, box, e, valid);
      // tangents: differences of w along the chain (file order is chain order)
      Vec3<Dd> ed[4];
      for (int k = 0; k < 4; ++k) {
        const int a = o - 2 + k, b = o - 1 + k;
        double t[3] = {0, 0, 0};
        if (valid[k])
          for (int d = 0; d < 3; ++d) t[d] = w[3 * a + d] - w[3 * b + d];
        ed[k] = Vec3<Dd>{{e[k].x, t[0]}, {e[k].y, t[1]}, {e[k].z, t[2]}};
      }
      const double* cd = T.chainD[set];
      const Dd cb[2] = {{cd[0], 0.0}, {cd[1], 0.0}};
      const Dd cn[2] = {{cd[2], 0.0}, {cd[3], 0.0}};
      Vec3<Dd> fbond{{0, 0}, {0, 0}, {0, 0}}, fbend{{0, 0}, {0, 0}, {0, 0}};
      if (valid[1]) bond_term<Dd>(ed[1], cb, Dd{-1.0, 0.0}, fbond);
      if (valid[2]) bond_term<Dd>(ed[2], cb, Dd{1.0, 0.0}, fbond);
      if (valid[0] && valid[1]) bend_term<Dd>(ed[0], ed[1], cn, 2, fbend);
      if (valid[1] && valid[2]) bend_term<Dd>(ed[1], ed[2], cn, 1, fbend);
      if (valid[2] && valid[3]) bend_term<Dd>(ed[2], ed[3], cn, 0, fbend);
      F[0] += fbond.x.v + fbend.x.v;
      F[1] += fbond.y.v + fbend.y.v;
      F[2] += fbond.z.v + fbend.z.v;
      K[0] += fbond.x.t + fbend.x.t;
      K[1] += fbond.y.t + fbend.y.t;
      K[2] += fbond.z.t + fbend.z.t;
      // dF/dk with unit constants (the forces are linear in k)
      const double ub[2] = {cd[0], 1.0}, un[2] = {cd[2], 1.0};
      Vec3<double> f1{0, 0, 0}, f2{0, 0, 0};
      if (valid[1]) bond_term<double>(e[1], ub, -1.0, f1);
      if (valid[2]) bond_term<double>(e[2], ub, 1.0, f1);
      if (valid[0] && valid[1]) bend_term<double>(e[0], e[1], un, 2, f2);
      if (valid[1] && valid[2]) bend_term<double>(e[1], e[2], un, 1, f2);
      if (valid[2] && valid[3]) bend_term<double>(e[2], e[3], un, 0, f2);
      // energies owned by the first bead of each bond / bend
      double ub_u = 0.0, un_u = 0.0;
      if (valid[2]) ub_u = bond_pot(e[2], ub);
      if (valid[2] && valid[3]) un_u = bend_pot(e[2], e[3], un);
      gJ = invT * (cd[1] * ub_u + cd[3] * un_u);
      g1 = dt * (wi[0] * f1.x + wi[1] * f1.y + wi[2] * f1.z) + invT * ub_u;
      g2 = dt * (wi[0] * f2.x + wi[1] * f2.y + wi[2] * f2.z) + invT * un_u;
    }
    const double damp = 1.0 - rp.gamma * dt;
    for (int d = 0; d < 3; ++d) {
      const double xb = xbar[3 * o + d] + dt * K[d] - invT * F[d];
      const double hb = damp * wi[d];
      xbar[3 * o + d] = xb;
      hbar[3 * o + d] = hb;
      w_next[3 * o + d] = hb + dt * xb;
    }
  }
  gJ = warp_sum(gJ);
  g1 = warp_sum(g1);
  g2 = warp_sum(g2);
  if ((threadIdx.x & 31) == 0) {
    if (gJ != 0.0) atomicAdd(&acc->J, gJ);
    if (g1 != 0.0) atomicAdd(&acc->grad[1], g1);
    if (g2 != 0.0) atomicAdd(&acc->grad[2], g2);
  }
}

// (K w)_i of the full conservative force at the current positions, file
// order, for a caller-supplied w: the pair part from k_adj_pair (kw) plus
// the CHAIN part, written to out (3n).
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_adj_hvp_out(DevPtrs P, int cur, const double* w, const double* kw,
                                                        double* out) {
  const int i = blockIdx.x * kBlock + threadIdx.x;
  if (i >= P.n) return;
  const Tables& T = *P.tab;
  const RepState& rs = P.rs[rep_of(P, i)];
  const double box[3] = {rs.box[0], rs.box[1], rs.box[2]};
  const int o = P.orig[i];
  double K[3] = {kw[i], kw[i + P.n], kw[i + 2 * P.n]};
  const int ci = P.cinfo[i];
  if (ci < 0 && !(ci & 0x40000000)) {
    const int p = ci & 0xfff, len = (ci >> 12) & 0xfff, set = (ci >> 24) & 0x1f;
    Vec3<double> e[4];
    bool valid[4];
    chain_vectors<MIXED, double>(P, cur, i, p, len, box, e, valid);
    Vec3<Dd> ed[4];
    for (int k = 0; k < 4; ++k) {
      const int a = o - 2 + k, b = o - 1 + k;
      double t[3] = {0, 0, 0};
      if (valid[k])
        for (int d = 0; d < 3; ++d) t[d] = w[3 * a + d] - w[3 * b + d];
      ed[k] = Vec3<Dd>{{e[k].x, t[0]}, {e[k].y, t[1]}, {e[k].z, t[2]}};
    }
    const double* cd = T.chainD[set];
    const Dd cb[2] = {{cd[0], 0.0}, {cd[1], 0.0}};
    const Dd cn[2] = {{cd[2], 0.0}, {cd[3], 0.0}};
    Vec3<Dd> f{{0, 0}, {0, 0}, {0, 0}};
    if (valid[1]) bond_term<Dd>(ed[1], cb, Dd{-1.0, 0.0}, f);
    if (valid[2]) bond_term<Dd>(ed[2], cb, Dd{1.0, 0.0}, f);
    if (valid[0] && valid[1]) bend_term<Dd>(ed[0], ed[1], cn, 2, f);
    if (valid[1] && valid[2]) bend_term<Dd>(ed[1], ed[2], cn, 1, f);
    if (valid[2] && valid[3]) bend_term<Dd>(ed[2], ed[3], cn, 0, f);
    K[0] += f.x.t;
    K[1] += f.y.t;
    K[2] += f.z.t;
  }
  for (int d = 0; d < 3; ++d) out[3 * o + d] = K[d];
}

}  // namespace smd
