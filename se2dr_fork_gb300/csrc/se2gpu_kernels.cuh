// se2gpu_kernels.cuh -- fused explicit SEM step for sm_103a.
//
// One launch advances the whole mesh by one Newmark (beta = 0, gamma = 1/2)
// step of se2wave.c:4722-4775:
//
//   u' = u + dt v + dt^2/2 a,  v* = v + dt/2 a               (4726-4730)
//   f  = K(u') + sum_s stf_s(t) g_s                           (4733-4739, 1285-1429, 3470-3497)
//   a' = f / M,  v' = v* + dt/2 a'                            (4742-4745)
//
// Work decomposition.  A CTA owns a rectangle of GLL nodes: the nodes of a tile
// of TE x TE elements, minus the node line shared with the next tile.  The
// nodes on its left/bottom boundary line also receive forces from the element
// column/row of the neighbouring tile, so the CTA additionally evaluates that
// one-element halo (it reads, but never writes, the halo nodes).  Every owned
// node then sums the contributions of the 1, 2 or 4 elements touching it in
// ascending element order -- the order in which the reference's
// VecSetValues(ADD) loop (1417) accumulates them -- so there are no atomics and
// results are deterministic.  Fields are double-buffered (read the old state,
// write the new), so halo reads never race with the neighbour's writes.
//
// Phases (all in shared memory):
//   1. load u, v, a (+ Kahan terms) of the node region, apply the predictor,
//      keep u' for the region and v* for the owned nodes;
//   2. strain -> Hooke stress at every GLL point of every element of tile+halo
//      (tensor-product / sum-factorised gradient);
//   3. weak divergence at the owned nodes, ordered element sum, source
//      injection, a' = f/M, corrector, store.
//
// FP64 mode reproduces the reference's floating-point operations exactly: the
// reference's dense sums over all npe basis functions only add exact zeros
// outside the tensor row/column of a point, so restricting each sum to the
// row/column while keeping its order, and keeping the products
// dN_dx = (1/J00) * dN_dxi, fac = detJ * w_q and -fac * (...), gives the same
// bits.  Every operation is __dmul_rn/__dadd_rn/__ddiv_rn (never contracted
// into an FMA).
//
// An extra CTA (blockIdx.x == number of tiles) samples the receivers from the
// OLD state: the state after the previous step, i.e. RecordUVA of that step.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace se2 {

template <typename T> struct Vec2;
template <> struct Vec2<double> { typedef double2 type; };
template <> struct Vec2<float> { typedef float2 type; };

template <typename T>
struct StepParams {
  int mx, my, nx_g, ny_g;     // elements, nodes per row/column
  int ntx, nty;               // tile grid
  int mode;                   // 0: time step, 1: internal force only (u_in -> f_out)
  const typename Vec2<T>::type *u_in, *v_in, *a_in, *cu_in, *cv_in;
  typename Vec2<T>::type *u_out, *v_out, *a_out, *cu_out, *cv_out, *f_out;
  const T *mass;              // FP64: lumped mass (divide); FP32: its reciprocal (multiply)
  const T *lam, *mu;          // per cell
  const T *J00, *J11, *iJ00, *iJ11;
  const T *D, *wq;            // (P+1)^2 tables in the compute type
  T c_dt, c_u, c_v;           // dt, 0.5*dt*dt, 0.5*dt (computed on the host as in se2wave.c:4726-4745)
  int nsrc;
  const int *src_elem;
  const T *src_vals;          // [nsrc][2*npe]
  const double *stf;          // this step's stf value per source
  int record, nrec;
  const int *rec_node, *rec_elem, *rec_gll;
  const double *Dd, *iJ00d, *iJ11d;  // FP64 tables for the receiver curl
  double *trace_row;          // [nrec*7] row for the sampled (old) state
};

// tile geometry (elements per tile edge) per degree
template <int P> struct Tile { static constexpr int TE = (P == 1) ? 32 : (P == 2) ? 16 : (P == 3) ? 11 : (P == 4) ? 8
                                                       : (P == 5) ? 6 : (P == 6) ? 5 : 4; };

// shared-memory carve, identical on host and device
struct Smem {
  size_t U, V, CU, CV, S, Dx, Dy, W, D, Nf, total;
};
__host__ __device__ inline size_t se2_align16(size_t x) { return (x + 15) & ~size_t(15); }
template <int P, typename T, bool KAHAN>
__host__ __device__ inline Smem smem_layout()
{
  constexpr int TE = Tile<P>::TE, N1 = P + 1, NPE = N1 * N1;
  constexpr int RW = (TE + 1) * P + 1;
  constexpr int NE = (TE + 1) * (TE + 1);
  constexpr int OW = TE * P + 1;
  Smem s;
  size_t o = 0;
  s.U = o;  o = se2_align16(o + sizeof(T) * 2 * RW * RW);
  s.V = o;  o = se2_align16(o + sizeof(T) * 2 * OW * OW);
  s.CU = o; o = se2_align16(o + (KAHAN ? sizeof(T) * 2 * OW * OW : 0));
  s.CV = o; o = se2_align16(o + (KAHAN ? sizeof(T) * 2 * OW * OW : 0));
  s.S = o;  o = se2_align16(o + sizeof(T) * 3 * NE * NPE);
  s.Dx = o; o = se2_align16(o + sizeof(T) * (TE + 1) * NPE);
  s.Dy = o; o = se2_align16(o + sizeof(T) * (TE + 1) * NPE);
  s.W = o;  o = se2_align16(o + sizeof(T) * NPE);
  s.D = o;  o = se2_align16(o + sizeof(T) * NPE);
  // FP64: -(detJ * w_q) per element and point, the factor of every divergence term, where
  // the table still leaves room for 2 CTAs per SM (otherwise it is formed per term)
  const size_t nf = (sizeof(T) == 8) ? sizeof(T) * NE * NPE : 0;
  s.Nf = o;
  if (nf && 2 * (se2_align16(o + nf) + 1024) <= 233472) o = se2_align16(o + nf);
  s.total = o;
  return s;
}

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

// Kahan summation of an increment into a running value with compensation c
__device__ __forceinline__ void kahan_add(float &s, float &c, float inc)
{
  const float y = inc - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// receivers, sampled from the *_in state (se2wave.c:2908-2962)
template <int P, typename T>
__device__ void sample_receivers(const StepParams<T> &prm)
{
  constexpr int N1 = P + 1;
  for (int r = threadIdx.x; r < prm.nrec; r += blockDim.x) {
    const int nid = prm.rec_node[r], eid = prm.rec_elem[r], g = prm.rec_gll[r];
    const auto u = prm.u_in[nid], v = prm.v_in[nid], a = prm.a_in[nid];
    double *o = prm.trace_row + 7 * r;
    o[0] = (double)u.x; o[1] = (double)u.y;
    o[2] = (double)v.x; o[3] = (double)v.y;
    o[4] = (double)a.x; o[5] = (double)a.y;
    const int ex = eid % prm.mx, ey = eid / prm.mx, ga = g % N1, gb = g / N1;
    const double ix = prm.iJ00d[ex], iy = prm.iJ11d[ey];
    double dvydx = 0.0, dvxdy = 0.0;
    // sum over the element's basis in ascending order; only the row (for d/dx)
    // and column (for d/dy) through the sampled point are non-zero
    for (int kb = 0; kb < N1; kb++) {
      const size_t n = (size_t)(ey * P + kb) * prm.nx_g + (size_t)(ex * P + ga);
      dvxdy = add(dvxdy, mul(mul(iy, prm.Dd[gb * N1 + kb]), (double)prm.v_in[n].x));
    }
    for (int ka = 0; ka < N1; ka++) {
      const size_t n = (size_t)(ey * P + gb) * prm.nx_g + (size_t)(ex * P + ka);
      dvydx = add(dvydx, mul(mul(ix, prm.Dd[ga * N1 + ka]), (double)prm.v_in[n].y));
    }
    o[6] = __dadd_rn(dvydx, -dvxdy);
  }
}

template <int P, typename T, bool KAHAN>
__global__ void __launch_bounds__(256)
step_kernel(const StepParams<T> prm)
{
  typedef typename Vec2<T>::type T2;
  constexpr bool F64 = (sizeof(T) == 8);
  constexpr int TE = Tile<P>::TE, N1 = P + 1, NPE = N1 * N1;
  constexpr int RWMAX = (TE + 1) * P + 1;
  constexpr int NEMAX = (TE + 1) * (TE + 1);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Smem L = smem_layout<P, T, KAHAN>();
  T2 *sU = reinterpret_cast<T2 *>(smem_raw + L.U);
  T2 *sV = reinterpret_cast<T2 *>(smem_raw + L.V);
  T2 *sCU = reinterpret_cast<T2 *>(smem_raw + L.CU);
  T2 *sCV = reinterpret_cast<T2 *>(smem_raw + L.CV);
  T *sSxx = reinterpret_cast<T *>(smem_raw + L.S);
  T *sSyy = sSxx + NEMAX * NPE;
  T *sSxy = sSyy + NEMAX * NPE;
  T *sDx = reinterpret_cast<T *>(smem_raw + L.Dx);
  T *sDy = reinterpret_cast<T *>(smem_raw + L.Dy);
  T *sW = reinterpret_cast<T *>(smem_raw + L.W);
  T *sD = reinterpret_cast<T *>(smem_raw + L.D);
  T *sNf = reinterpret_cast<T *>(smem_raw + L.Nf);

  const int ntiles = prm.ntx * prm.nty;
  if ((int)blockIdx.x >= ntiles) {
    if (prm.record) sample_receivers<P, T>(prm);
    return;
  }
  const int mx = prm.mx, my = prm.my, nx_g = prm.nx_g;
  const int tx = blockIdx.x % prm.ntx, ty = blockIdx.x / prm.ntx;
  const int ex0 = tx * TE, ex1 = min(ex0 + TE, mx);
  const int ey0 = ty * TE, ey1 = min(ey0 + TE, my);
  const int EX0 = max(ex0 - 1, 0), EY0 = max(ey0 - 1, 0);
  const int NEX = ex1 - EX0, NEY = ey1 - EY0;
  const int RX0 = EX0 * P, RY0 = EY0 * P;
  const int RW = NEX * P + 1, RH = NEY * P + 1;
  const int X0 = ex0 * P, Y0 = ey0 * P;
  const int OW = (ex1 - ex0) * P + (ex1 == mx ? 1 : 0);
  const int OH = (ey1 - ey0) * P + (ey1 == my ? 1 : 0);
  const bool step = (prm.mode == 0);

  // ---- phase 1: load + predictor -------------------------------------
  for (int idx = threadIdx.x; idx < RW * RH; idx += blockDim.x) {
    const int ry = idx / RW, rx = idx - ry * RW;
    const int X = RX0 + rx, Y = RY0 + ry;
    const size_t n = (size_t)Y * nx_g + X;
    T2 up = prm.u_in[n];
    if (step) {
      const T2 v = prm.v_in[n], a = prm.a_in[n];
      const bool own = (X >= X0) && (X < X0 + OW) && (Y >= Y0) && (Y < Y0 + OH);
      T2 vs;
      if constexpr (F64) {
        // VecAXPY(u,dt,v); VecAXPY(u,0.5*dt*dt,a); VecAXPY(v,0.5*dt,a)
        up.x = add(add(up.x, mul(prm.c_dt, v.x)), mul(prm.c_u, a.x));
        up.y = add(add(up.y, mul(prm.c_dt, v.y)), mul(prm.c_u, a.y));
        vs.x = add(v.x, mul(prm.c_v, a.x));
        vs.y = add(v.y, mul(prm.c_v, a.y));
      } else if constexpr (KAHAN) {
        T2 cu = prm.cu_in[n];
        kahan_add(up.x, cu.x, fmaf(prm.c_dt, v.x, prm.c_u * a.x));
        kahan_add(up.y, cu.y, fmaf(prm.c_dt, v.y, prm.c_u * a.y));
        if (own) {
          T2 cv = prm.cv_in[n];
          vs = v;
          kahan_add(vs.x, cv.x, prm.c_v * a.x);
          kahan_add(vs.y, cv.y, prm.c_v * a.y);
          const int o = (Y - Y0) * OW + (X - X0);
          sCU[o] = cu;
          sCV[o] = cv;
        }
      } else {
        up.x = fmaf(prm.c_dt, v.x, fmaf(prm.c_u, a.x, up.x));
        up.y = fmaf(prm.c_dt, v.y, fmaf(prm.c_u, a.y, up.y));
        vs.x = fmaf(prm.c_v, a.x, v.x);
        vs.y = fmaf(prm.c_v, a.y, v.y);
      }
      if (own) sV[(Y - Y0) * OW + (X - X0)] = vs;
    }
    sU[idx] = up;
  }
  // tables: FP64 keeps the reference's scaled derivatives dN_dx = (1/J00) * D per element column/row
  for (int i = threadIdx.x; i < NPE; i += blockDim.x) { sW[i] = prm.wq[i]; sD[i] = prm.D[i]; }
  if constexpr (F64) {
    for (int i = threadIdx.x; i < NEX * NPE; i += blockDim.x) sDx[i] = mul(prm.iJ00[EX0 + i / NPE], prm.D[i % NPE]);
    for (int i = threadIdx.x; i < NEY * NPE; i += blockDim.x) sDy[i] = mul(prm.iJ11[EY0 + i / NPE], prm.D[i % NPE]);
    // the same value the divergence would form per term: -(J00 J11) * w_q, operand order kept
    if (L.total > L.Nf)
    for (int i = threadIdx.x; i < NEX * NEY * NPE; i += blockDim.x) {
      const int el = i / NPE, q = i - el * NPE, ecy = el / NEX, ecx = el - ecy * NEX;
      sNf[i] = -mul(mul(prm.J00[EX0 + ecx], prm.J11[EY0 + ecy]), prm.wq[q]);
    }
  }
  __syncthreads();

  // ---- phase 2: stress at every GLL point of tile + halo -------------
  // FP64 walks the points row by row of their element (qj outermost), so the
  // shear-strain sum's branch on qj is the same for nearly every thread of a warp
  const int NEL = NEX * NEY;
  for (int it = threadIdx.x; it < NEL * NPE; it += blockDim.x) {
    int el, q;
    if constexpr (F64) {
      const int qj_ = it / (NEL * N1), r = it - qj_ * (NEL * N1);
      el = r / N1;
      q = (r - el * N1) + qj_ * N1;
    } else {
      el = it / NPE;
      q = it - el * NPE;
    }
    const int idx = el * NPE + q;
    const int ecy = el / NEX, ecx = el - ecy * NEX;
    const int qj = q / N1, qi = q - qj * N1;
    const int ex = EX0 + ecx, ey = EY0 + ecy;
    const T2 *ue = sU + (ecy * P) * RW + ecx * P;   // local node (0,0)
    const size_t cell = (size_t)ey * mx + ex;
    const T lam = prm.lam[cell], mu = prm.mu[cell];
    if constexpr (F64) {
      const double *dx = sDx + ecx * NPE + qi * N1;  // dN/dx of basis (ia, qj) at q
      const double *dy = sDy + ecy * NPE + qj * N1;  // dN/dy of basis (qi, ib) at q
      double e0 = 0.0, e1 = 0.0, e2 = 0.0;
#pragma unroll
      for (int ia = 0; ia < N1; ia++) e0 = add(e0, mul(dx[ia], ue[qj * RW + ia].x));
#pragma unroll
      for (int ib = 0; ib < N1; ib++) e1 = add(e1, mul(dy[ib], ue[ib * RW + qi].y));
      // shear strain: basis index ascending = column below, row, column above
#pragma unroll
      for (int ib = 0; ib < N1; ib++) {
        if (ib < qj || ib > qj) {
          e2 = add(e2, mul(dy[ib], ue[ib * RW + qi].x));
        } else {
#pragma unroll
          for (int ia = 0; ia < N1; ia++) {
            double t = mul(dx[ia], ue[qj * RW + ia].y);
            if (ia == qi) t = add(t, mul(dy[qj], ue[qj * RW + qi].x));
            e2 = add(e2, t);
          }
        }
      }
      const double c11 = add(mul(2.0, mu), lam);
      sSxx[idx] = add(mul(c11, e0), mul(lam, e1));
      sSyy[idx] = add(mul(lam, e0), mul(c11, e1));
      sSxy[idx] = mul(mu, e2);
    } else {
      float gx_ux = 0.f, gx_uy = 0.f, gy_ux = 0.f, gy_uy = 0.f;
#pragma unroll
      for (int k = 0; k < N1; k++) {
        const float dxk = sD[qi * N1 + k], dyk = sD[qj * N1 + k];
        const float2 ur = ue[qj * RW + k];   // row through q
        const float2 uc = ue[k * RW + qi];   // column through q
        gx_ux = fmaf(dxk, ur.x, gx_ux);
        gx_uy = fmaf(dxk, ur.y, gx_uy);
        gy_ux = fmaf(dyk, uc.x, gy_ux);
        gy_uy = fmaf(dyk, uc.y, gy_uy);
      }
      const float ix = prm.iJ00[ex], iy = prm.iJ11[ey];
      const float e0 = ix * gx_ux, e1 = iy * gy_uy, e2 = fmaf(ix, gx_uy, iy * gy_ux);
      const float c11 = fmaf(2.f, mu, lam);
      const float nfac = -(prm.J00[ex] * prm.J11[ey]) * sW[q];
      sSxx[idx] = nfac * fmaf(c11, e0, lam * e1);
      sSyy[idx] = nfac * fmaf(lam, e0, c11 * e1);
      sSxy[idx] = nfac * (mu * e2);
    }
  }
  __syncthreads();

  // ---- phase 3: divergence, ordered element sum, source, update -------
  // FP64 takes the nodes on element-column lines (2 elements along x) first and the
  // others after, each group ordered by the node's row within its element (which
  // decides the branches of the element sums) and then by row and column, so a warp's
  // threads loop over the same elements and take the same branches
  const int NC1 = (OW + P - 1) / P, NC0 = OW - NC1;   // columns on / between element lines
  for (int o = threadIdx.x; o < OW * OH; o += blockDim.x) {
    int oy, ox;
    if constexpr (F64) {
      const bool on = o < NC1 * OH;
      const int nc = on ? NC1 : NC0;
      int r = on ? o : o - NC1 * OH, b = 0;
      for (; b < P - 1; b++) {          // rows oy = b, b + P, ... of the tile
        const int nb = nc * ((OH - b + P - 1) / P);
        if (r < nb) break;
        r -= nb;
      }
      const int row = r / nc, col = r - row * nc;
      oy = row * P + b;
      if (on) {
        ox = col * P;
      } else {
        constexpr int PM = (P > 1) ? P - 1 : 1;   // interior nodes per element along x (degree 1: none)
        ox = (col / PM) * P + (col % PM) + 1;
      }
    } else {
      oy = o / OW;
      ox = o - oy * OW;
    }
    const int X = X0 + ox, Y = Y0 + oy;
    T fx = 0, fy = 0;
    const int eyA = (Y % P == 0) ? Y / P - 1 : Y / P, exA = (X % P == 0) ? X / P - 1 : X / P;
    const int eyB = Y / P, exB = X / P;
    for (int ey = eyA; ey <= eyB; ey++) {
      if (ey < 0 || ey >= my) continue;
      for (int ex = exA; ex <= exB; ex++) {
        if (ex < 0 || ex >= mx) continue;
        const int ecx = ex - EX0, ecy = ey - EY0, el = ecy * NEX + ecx;
        const int a = X - ex * P, b = Y - ey * P;
        const T *Sxx = sSxx + el * NPE, *Syy = sSyy + el * NPE, *Sxy = sSxy + el * NPE;
        if constexpr (F64) {
          const bool nft = L.total > L.Nf;   // the factor table exists (room for 2 CTAs)
          const double *nfe = sNf + el * NPE;
          const double detJ = nft ? 0.0 : mul(prm.J00[ex], prm.J11[ey]);
          const double *dx = sDx + ecx * NPE, *dy = sDy + ecy * NPE;
          double gx = 0.0, gy = 0.0;
          // quadrature points ascending: column below b, row b, column above b
#pragma unroll
          for (int qj = 0; qj < N1; qj++) {
            if (qj != b) {
              const int q = a + qj * N1;
              const double nf = nft ? nfe[q] : -mul(detJ, sW[q]);
              const double dNy = dy[qj * N1 + b];
              gx = add(gx, mul(nf, mul(dNy, Sxy[q])));
              gy = add(gy, mul(nf, mul(dNy, Syy[q])));
            } else {
#pragma unroll
              for (int qi = 0; qi < N1; qi++) {
                const int q = qi + b * N1;
                const double nf = nft ? nfe[q] : -mul(detJ, sW[q]);
                const double dNx = dx[qi * N1 + a];
                double tx, ty;
                if (qi == a) {
                  const double dNy = dy[b * N1 + b];
                  tx = add(mul(dNx, Sxx[q]), mul(dNy, Sxy[q]));
                  ty = add(mul(dNy, Syy[q]), mul(dNx, Sxy[q]));
                } else {
                  tx = mul(dNx, Sxx[q]);
                  ty = mul(dNx, Sxy[q]);
                }
                gx = add(gx, mul(nf, tx));
                gy = add(gy, mul(nf, ty));
              }
            }
          }
          fx = add(fx, gx);
          fy = add(fy, gy);
        } else {
          float rx = 0.f, ry = 0.f, cx = 0.f, cy = 0.f;
#pragma unroll
          for (int k = 0; k < N1; k++) {
            const float dxa = sD[k * N1 + a], dyb = sD[k * N1 + b];
            rx = fmaf(dxa, Sxx[k + b * N1], rx);
            ry = fmaf(dxa, Sxy[k + b * N1], ry);
            cx = fmaf(dyb, Sxy[a + k * N1], cx);
            cy = fmaf(dyb, Syy[a + k * N1], cy);
          }
          const float ix = prm.iJ00[ex], iy = prm.iJ11[ey];
          fx += fmaf(ix, rx, iy * cx);
          fy += fmaf(ix, ry, iy * cy);
        }
      }
    }
    const size_t n = (size_t)Y * nx_g + X;
    if (!step) {
      T2 f; f.x = fx; f.y = fy;
      prm.f_out[n] = f;
      continue;
    }
    // source injection: g = sum_s stf_s * g_s, then f + 1.0*g
    T gsx = 0, gsy = 0;
    for (int s = 0; s < prm.nsrc; s++) {
      const int se = prm.src_elem[s], sx = se % mx, sy = se / mx;
      const int a = X - sx * P, b = Y - sy * P;
      if (a >= 0 && a <= P && b >= 0 && b <= P) {
        const T val = (T)prm.stf[s];
        const T *sv = prm.src_vals + (size_t)s * 2 * NPE + 2 * (a + b * N1);
        if constexpr (F64) { gsx = add(gsx, mul(val, sv[0])); gsy = add(gsy, mul(val, sv[1])); }
        else { gsx = fmaf(val, sv[0], gsx); gsy = fmaf(val, sv[1], gsy); }
      }
    }
    const int ol = (Y - Y0) * OW + (X - X0);
    const int rl = (Y - RY0) * RW + (X - RX0);
    T2 an, vn = sV[ol];
    if constexpr (F64) {
      const double m = prm.mass[n];
      an.x = __ddiv_rn(add(fx, gsx), m);
      an.y = __ddiv_rn(add(fy, gsy), m);
      vn.x = add(vn.x, mul(prm.c_v, an.x));
      vn.y = add(vn.y, mul(prm.c_v, an.y));
    } else {
      const float minv = prm.mass[n];
      an.x = (fx + gsx) * minv;
      an.y = (fy + gsy) * minv;
      if constexpr (KAHAN) {
        T2 cv = sCV[ol];
        kahan_add(vn.x, cv.x, prm.c_v * an.x);
        kahan_add(vn.y, cv.y, prm.c_v * an.y);
        prm.cv_out[n] = cv;
        prm.cu_out[n] = sCU[ol];
      } else {
        vn.x = fmaf(prm.c_v, an.x, vn.x);
        vn.y = fmaf(prm.c_v, an.y, vn.y);
      }
    }
    prm.u_out[n] = sU[rl];
    prm.v_out[n] = vn;
    prm.a_out[n] = an;
  }
}

// standalone receiver sampling (used after the last step of a block)
template <int P, typename T>
__global__ void record_kernel(const StepParams<T> prm)
{
  sample_receivers<P, T>(prm);
}

// ---- norms: per-block partials, then a single-block fixed-order finish ----
template <typename T>
__global__ void norms_partial(const T *u, const T *v, long n, double *part)
{
  __shared__ double s[6][256];
  double umax = -1.0e308, umin = 1.0e308, uss = 0.0, vmax = -1.0e308, vmin = 1.0e308, vss = 0.0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double a = (double)u[i], b = (double)v[i];
    umax = fmax(umax, a); umin = fmin(umin, a); uss += a * a;
    vmax = fmax(vmax, b); vmin = fmin(vmin, b); vss += b * b;
  }
  s[0][threadIdx.x] = umax; s[1][threadIdx.x] = umin; s[2][threadIdx.x] = uss;
  s[3][threadIdx.x] = vmax; s[4][threadIdx.x] = vmin; s[5][threadIdx.x] = vss;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const int t = threadIdx.x;
      s[0][t] = fmax(s[0][t], s[0][t + w]); s[1][t] = fmin(s[1][t], s[1][t + w]); s[2][t] += s[2][t + w];
      s[3][t] = fmax(s[3][t], s[3][t + w]); s[4][t] = fmin(s[4][t], s[4][t + w]); s[5][t] += s[5][t + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

}  // namespace se2
