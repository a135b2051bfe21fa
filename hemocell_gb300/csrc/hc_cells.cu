// Cell kernels of the GB300 HemoCell step (sm_103a):
//   K2 spread          IBM phi2 force spreading with FORCE_LIMIT clamp; one
//                      vector atomic per node contribution (FP32); tags the
//                      stencil nodes for the interpolation
//   K3+K5 interp_advance  velocity interpolation from the tagged node
//                      velocities, Euler advance, nearest-node bin, wall deletion
//   K4 mechanics       RBC / PLT / WBC membrane forces, one CTA per cell
//   binning            tile CSR sorted by (tile, cell, vertex)
// Templated on T = double (plain form) or float (mixed form); positions are
// double in both forms.
#include <cmath>
#include <cstdint>

#include "hc_async.cuh"
#include "hc_d3q19.cuh"
#include "hc_posbits.h"

namespace hcd {

template <typename T>
__device__ __forceinline__ T tmax(T a, T b) {
  return a > b ? a : b;
}

// IBM phi2 kernel (core/immersedBoundaryMethod.h:37-41, :62-138).  The
// reference scans the 3x3x3 nodes around floor(p+0.5) and keeps the nonzero
// weights; phi2 vanishes beyond distance 1, so the kept nodes always lie in
// the 2x2x2 block {floor(p), floor(p)+1}^3, scanned here in the same
// (x, y, z) order.  Nodes off a non-periodic axis, zero weights and boundary
// nodes are skipped (slot node = -1); the weights are renormalised to one.
// FP64 evaluates phi2(p - q) exactly as the reference; FP32 takes the
// fractional part (float)(p - floor(p)) once, from the bits of the FP64
// coordinate (hc_posbits.h), and the rest in float.
template <typename T>
struct Kern {
  int node[8];  // the lattice holds fewer than 2^31 nodes (hc_create's size limit)
  T w[8];
};

template <typename T>
__device__ __forceinline__ void ibm_weights(const LbmView<T>& L, double px, double py, double pz, Kern<T>& K) {
  constexpr bool kF64 = sizeof(T) == 8;
  const double P[3] = {px, py, pz};
  const int dims[3] = {L.nx, L.ny, L.nz};
  T phi[3][2];
  int idx[3][2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    long long qi;
    if (kF64) {
      const double q0 = floor(P[a]);
      phi[a][0] = tmax(T(1) - T(fabs(P[a] - q0)), T(0));
      phi[a][1] = tmax(T(1) - T(fabs(P[a] - (q0 + 1.0))), T(0));
      qi = (long long)q0;
    } else {
      // floor(P) and the fraction (float)(P - floor(P)) from the bits of P,
      // the FP64 instructions only outside [1, 2^31)
      // A fraction within 2^-25 of one rounds to 1.0f; the lower node's
      // weight is then the rounded exact complement 1 - (P - floor(P)), not
      // zero, so that a vertex next to a wall keeps the FP64 form's
      // renormalised stencil.
      int qs;
      float w0, w1;
      if (hcpos::split_weights(P[a], qs, w0, w1)) {
        qi = qs;
      } else {
        const double q0 = floor(P[a]);
        const double fr = P[a] - q0;  // exact, as is 1 - fr
        w1 = (float)fr;
        w0 = w1 == 1.0f ? (float)(1.0 - fr) : 1.0f - w1;
        qi = (long long)q0;
      }
      phi[a][0] = (T)w0;
      phi[a][1] = (T)w1;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const long long q = qi + k;
      int wrapped;
      if (q < 0 || q >= dims[a]) {
        if (L.per[a]) {
          long long mm = q % dims[a];
          wrapped = (int)(mm < 0 ? mm + dims[a] : mm);
        } else {
          wrapped = -1;
        }
      } else {
        wrapped = (int)q;
      }
      idx[a][k] = wrapped;
    }
  }
  T total = T(0);
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int ax = s >> 2, ay = (s >> 1) & 1, az = s & 1;
    K.node[s] = -1;
    K.w[s] = T(0);
    if (idx[0][ax] < 0 || idx[1][ay] < 0 || idx[2][az] < 0) continue;
    const T w = phi[0][ax] * phi[1][ay] * phi[2][az];
    if (w == T(0)) continue;
    const int nd = idx[0][ax] + L.nx * (idx[1][ay] + L.ny * idx[2][az]);
    if (!HC_IN(L.status, nd, L.N) || L.flag[nd] != 0) continue;
    total += w;
    K.node[s] = nd;
    K.w[s] = w;
  }
  if (total > T(0)) {
    const T coeff = T(1) / total;
#pragma unroll
    for (int s = 0; s < 8; ++s) K.w[s] *= coeff;
  }
}

// ---------------------------------------------------------------------------
// K2: spreadParticleForce (core/hemoCellParticleField.cpp:841-863) with the
// FORCE_LIMIT clamp written back (:847-852); the stencil nodes are tagged
// with the step stamp so the interpolation evaluates only those nodes.
template <typename T>
__global__ void __launch_bounds__(256) k_spread(const LbmView<T> L, const VertexView<T> vv, const T f_limit) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vv.nvert || !vv.alive[vv.vcell[i]]) return;
  const uint32_t stamp = *L.stamp;
  const long long V = vv.V;
  T fx = vv.f[i], fy = vv.f[V + i], fz = vv.f[2 * V + i];
  T mag = fx * fx;
  mag += fy * fy;
  mag += fz * fz;
  mag = sqrt(mag);
  if (mag > f_limit) {
    const T s = f_limit / mag;
    fx *= s;
    fy *= s;
    fz *= s;
    vv.f[i] = fx;
    vv.f[V + i] = fy;
    vv.f[2 * V + i] = fz;
  }
  // the repulsion force is spread with the clamped force (:857-859)
  if (vv.frep_cell) {
    fx += vv.frep_cell[i];
    fy += vv.frep_cell[V + i];
    fz += vv.frep_cell[2 * V + i];
  }
  if (vv.frep_wall) {
    fx += vv.frep_wall[i];
    fy += vv.frep_wall[V + i];
    fz += vv.frep_wall[2 * V + i];
  }
  Kern<T> K;
  ibm_weights(L, vv.x[i], vv.x[V + i], vv.x[2 * V + i], K);
  T* F = const_cast<T*>(L.Fcur);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (K.node[j] < 0) continue;
    if (L.ntag) L.ntag[K.node[j]] = stamp;
    FieldLayout<T>::add(F, L.N, K.node[j], fx * K.w[j], fy * K.w[j], fz * K.w[j]);
  }
  pdl_trigger();
}

template <typename T>
cudaError_t launch_spread(const LbmView<T>& L, const VertexView<T>& vv, double f_limit, int bs, cudaStream_t s) {
  if (vv.nvert <= 0) return cudaSuccess;
  if (bs <= 0) bs = 128;
  return launch_kernel(k_spread<T>, dim3((vv.nvert + bs - 1) / bs), dim3(bs), 0, s, L.pdl, L, vv, (T)f_limit);
}

// ---------------------------------------------------------------------------
// CellInformation (helper/cellInfo.cpp:170-266), one CTA per cell: centroid,
// mean velocity, membrane area, enclosed volume (six-term sum over faces, on
// coordinates relative to the cell's vertex 0), largest distance between two
// of its vertices (stretch), bounding box.  out holds 16 doubles per cell:
// cx cy cz vx vy vz area volume stretch xmin xmax ymin ymax zmin zmax type
// (type -1 once the cell was deleted).
template <typename T>
__global__ void __launch_bounds__(256) k_cell_info(const VertexView<T> vv, const int* cell_type, const int* cell_voff,
                                                   const TypeDev* types, double* out) {
  __shared__ double red[32][16];
  const int cell = blockIdx.x;
  const TypeDev& t = types[cell_type[cell]];
  const int nv = t.nv, voff = cell_voff[cell];
  const long long V = vv.V;
  const double* X = vv.x;
  const double o[3] = {X[voff], X[V + voff], X[2 * V + voff]};
  double acc[16];
  for (int k = 0; k < 16; ++k) acc[k] = 0.0;
  acc[9] = acc[11] = acc[13] = 1e300;    // minima
  acc[10] = acc[12] = acc[14] = -1e300;  // maxima
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    for (int a = 0; a < 3; ++a) {
      const double p = X[a * V + voff + i];
      acc[a] += p;
      acc[3 + a] += (double)vv.v[a * V + voff + i];
      acc[9 + 2 * a] = fmin(acc[9 + 2 * a], p);
      acc[10 + 2 * a] = fmax(acc[10 + 2 * a], p);
    }
    double pi[3];
    for (int a = 0; a < 3; ++a) pi[a] = X[a * V + voff + i];
    for (int j = i + 1; j < nv; ++j) {
      double d2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        const double d = pi[a] - X[a * V + voff + j];
        d2 += d * d;
      }
      acc[8] = fmax(acc[8], d2);
    }
  }
  for (int k = threadIdx.x; k < t.nf; k += blockDim.x) {
    double v[3][3];
    for (int c = 0; c < 3; ++c)
      for (int a = 0; a < 3; ++a) v[c][a] = X[a * V + voff + t.tris[3 * k + c]] - o[a];
    const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
    const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                 cz = e1[0] * e2[1] - e1[1] * e2[0];
    acc[6] += 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    acc[7] += (-v[2][0] * v[1][1] * v[0][2] + v[1][0] * v[2][1] * v[0][2] + v[2][0] * v[0][1] * v[1][2] -
               v[0][0] * v[2][1] * v[1][2] - v[1][0] * v[0][1] * v[2][2] + v[0][0] * v[1][1] * v[2][2]) /
              6.0;
  }
  // block reduction: sums for 0-7, max for 8, 10, 12, 14, min for 9, 11, 13
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int k = 0; k < 15; ++k) {
    double x = acc[k];
    for (int off = 16; off > 0; off >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, off);
      x = k < 8 ? x + y : ((k == 9 || k == 11 || k == 13) ? fmin(x, y) : fmax(x, y));
    }
    if (lane == 0) red[wid][k] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[15];
    for (int k = 0; k < 15; ++k) {
      r[k] = red[0][k];
      for (int w = 1; w < nw; ++w)
        r[k] = k < 8 ? r[k] + red[w][k] : ((k == 9 || k == 11 || k == 13) ? fmin(r[k], red[w][k]) : fmax(r[k], red[w][k]));
    }
    double* dst = out + 16 * (size_t)cell;
    for (int a = 0; a < 3; ++a) {
      dst[a] = r[a] / nv;
      dst[3 + a] = r[3 + a] / nv;
    }
    dst[6] = r[6];
    dst[7] = r[7];
    dst[8] = sqrt(r[8]);
    for (int k = 9; k < 15; ++k) dst[k] = r[k];
    dst[15] = vv.alive[cell] ? (double)cell_type[cell] : -1.0;
  }
}

template <typename T>
cudaError_t launch_cell_info(const VertexView<T>& vv, const int* cell_type, const int* cell_voff, const TypeDev* types,
                             int ncells, double* out, cudaStream_t s) {
  if (ncells <= 0) return cudaSuccess;
  k_cell_info<T><<<ncells, 256, 0, s>>>(vv, cell_type, cell_voff, types, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Repulsion.  k_rep_bin bins every vertex of a live cell at its node
// int(x + 0.5) (core/hemoCellParticleField.cpp:153-156), wrapped on periodic
// axes, and keeps its position relative to that node.  k_repulsion then
// gathers, per vertex, over the 27 nodes around its own: vertices of other
// cells closer than the cutoff push with kc * (rc / d) along the separation,
// counted twice when they share the node (the reference visits a node's own
// pairs in both orders, :678-694), and boundary nodes closer than the wall
// cutoff push with kw * (rw / d) (:891-918).  Node offsets of at most one in
// each axis make the separation (x_p - q_p) - (x_b - q_b) - d exact in the
// working precision and take the periodic image.  Each node's vertices are
// visited in ascending index order so the sums are deterministic.
template <typename T>
__global__ void k_rep_bin(const LbmView<T> L, const VertexView<T> vv, const RepView<T> R) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vv.nvert) return;
  int q = -1;
  if (vv.alive[vv.vcell[i]]) {
    const long long V = vv.V;
    const double P[3] = {vv.x[i], vv.x[V + i], vv.x[2 * V + i]};
    const int n[3] = {L.nx, L.ny, L.nz};
    int c[3];
    T r[3];
    bool in = true;
    for (int a = 0; a < 3; ++a) {
      const double b = floor(P[a] + 0.5);
      r[a] = (T)(P[a] - b);
      long long v = (long long)b;
      if (L.per[a]) v = ((v % n[a]) + n[a]) % n[a];
      else if (v < 0 || v >= n[a]) in = false;
      c[a] = (int)v;
    }
    if (in) {
      q = c[0] + L.nx * (c[1] + L.ny * c[2]);
      for (int a = 0; a < 3; ++a) R.xr[a * V + i] = r[a];
      if (R.cnt) {
        const int s = atomicAdd(R.cnt + q, 1);
        if (s < REP_SLOTS) R.slot[(long long)q * REP_SLOTS + s] = i;
        else atomicOr(L.status, STATUS_REP_OVERFLOW);
      }
    }
  }
  R.vq[i] = q;
}

template <typename T>
__global__ void k_repulsion(const LbmView<T> L, const VertexView<T> vv, const RepView<T> R) {
  pdl_wait();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= vv.nvert) return;
  const long long V = vv.V;
  const int q0 = R.vq[p];
  T fc[3] = {T(0), T(0), T(0)}, fw[3] = {T(0), T(0), T(0)};
  if (q0 >= 0) {
    const int X0 = q0 % L.nx, Y0 = (q0 / L.nx) % L.ny, Z0 = q0 / (L.nx * L.ny);
    const T rp[3] = {R.xr[p], R.xr[V + p], R.xr[2 * V + p]};
    const int cp = vv.vcell[p];
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int d[3] = {dx, dy, dz};
          const int c0[3] = {X0, Y0, Z0}, n[3] = {L.nx, L.ny, L.nz};
          int c[3];
          bool out = false;
          for (int a = 0; a < 3; ++a) {
            c[a] = c0[a] + d[a];
            if (c[a] < 0 || c[a] >= n[a]) {
              if (L.per[a]) c[a] = c[a] < 0 ? c[a] + n[a] : c[a] - n[a];
              else out = true;
            }
          }
          if (out) continue;
          const int qb = c[0] + L.nx * (c[1] + L.ny * c[2]);
          if (R.fcell) {
            const int cnt = min(R.cnt[qb], REP_SLOTS);
            const int* sl = R.slot + (long long)qb * REP_SLOTS;
            const T mult = (dx == 0 && dy == 0 && dz == 0) ? T(2) : T(1);
            int last = -1;
            for (int k = 0; k < cnt; ++k) {
              int b = 0x7fffffff;
              for (int m = 0; m < cnt; ++m) {
                const int v = sl[m];
                if (v > last && v < b) b = v;
              }
              last = b;
              if (vv.vcell[b] == cp) continue;
              T dv[3];
              for (int a = 0; a < 3; ++a) dv[a] = (rp[a] - R.xr[a * V + b]) - T(d[a]);
              const T dist = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
              if (dist < R.rc) {
                const T s = mult * R.kc * (R.rc / dist) / dist;
                for (int a = 0; a < 3; ++a) fc[a] += dv[a] * s;
              }
            }
          }
          if (R.fwall && R.bnode[qb]) {
            T dv[3];
            for (int a = 0; a < 3; ++a) dv[a] = rp[a] - T(d[a]);
            const T dist = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
            if (dist < R.rw) {
              const T s = R.kw * (R.rw / dist) / dist;
              for (int a = 0; a < 3; ++a) fw[a] += dv[a] * s;
            }
          }
        }
  }
  for (int a = 0; a < 3; ++a) {
    if (R.fcell) R.fcell[a * V + p] = fc[a];
    if (R.fwall) R.fwall[a * V + p] = fw[a];
  }
}

template <typename T>
cudaError_t launch_repulsion(const LbmView<T>& L, const VertexView<T>& vv, const RepView<T>& R, cudaStream_t s) {
  if (vv.nvert <= 0) return cudaSuccess;
  const int g = (vv.nvert + 255) / 256;
  cudaError_t e = launch_kernel(k_rep_bin<T>, dim3(g), dim3(256), 0, s, L.pdl, L, vv, R);
  if (e != cudaSuccess) return e;
  return launch_kernel(k_repulsion<T>, dim3(g), dim3(256), 0, s, L.pdl, L, vv, R);
}

// Tag the stencil nodes of every vertex (the interpolation run as a stage
// of its own, without the spread of the same step).
template <typename T>
__global__ void k_mark_nodes(const LbmView<T> L, const VertexView<T> vv) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vv.nvert || !vv.alive[vv.vcell[i]]) return;
  const uint32_t stamp = *L.stamp;
  Kern<T> K;
  ibm_weights(L, vv.x[i], vv.x[vv.V + i], vv.x[2 * vv.V + i], K);
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (K.node[j] >= 0 && L.ntag) L.ntag[K.node[j]] = stamp;
}
template <typename T>
cudaError_t launch_mark_nodes(const LbmView<T>& L, const VertexView<T>& vv, cudaStream_t s) {
  if (vv.nvert <= 0) return cudaSuccess;
  return launch_kernel(k_mark_nodes<T>, dim3((vv.nvert + 255) / 256), dim3(256), 0, s, L.pdl, L, vv);
}

// External vertex forces (HemoCellStretch::applyForce adds them to the
// vertex force right before the spread, helper/hemoCellStretch.cpp:63-78).
template <typename T>
__global__ void k_add_vertex_forces(const VertexView<T> vv, const int* ids, const double* fext, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i = ids[k];
  if (i < 0 || i >= vv.nvert) return;
  vv.f[i] += (T)fext[3 * k];
  vv.f[vv.V + i] += (T)fext[3 * k + 1];
  vv.f[2 * vv.V + i] += (T)fext[3 * k + 2];
}
template <typename T>
cudaError_t launch_add_vertex_forces(const VertexView<T>& vv, const int* ids, const double* fext, int n,
                                     cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_add_vertex_forces<T><<<(n + 127) / 128, 128, 0, s>>>(vv, ids, fext, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// K3+K5: interpolateFluidVelocity (core/hemoCellParticleField.cpp:819-839)
// from the node velocities of this step (L.unode), advanceParticles
// (:566-588, core/hemoCellParticle.h:188-203) and the per-vertex bin of
// update_pg (:137-168).  Thread 0 advances the device step stamp; no thread
// of this kernel reads it.
template <typename T>
__global__ void __launch_bounds__(256) k_interp_advance(const LbmView<T> L, const VertexView<T> vv, const TileGrid tg,
                                                        const int do_interp, const int do_advance) {
  pdl_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *L.stamp += 1;
  if (i >= vv.nvert) return;
  const int cell = vv.vcell[i];
  if (!vv.alive[cell]) {
    vv.vnode[i] = -1;
    vv.vtile[i] = -1;
    return;
  }
  const long long V = vv.V;
  double px = vv.x[i], py = vv.x[V + i], pz = vv.x[2 * V + i];
  T vx, vy, vz;
  if (do_interp) {
    Kern<T> K;
    ibm_weights(L, px, py, pz, K);
    vx = T(0);
    vy = T(0);
    vz = T(0);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (K.node[j] < 0) continue;
      T ux, uy, uz;
      FieldLayout<T>::load(L.unode, L.N, K.node[j], ux, uy, uz);
      vx += ux * K.w[j];
      vy += uy * K.w[j];
      vz += uz * K.w[j];
    }
    vv.v[i] = vx;
    vv.v[V + i] = vy;
    vv.v[2 * V + i] = vz;
    if (!(isfinite(vx) && isfinite(vy) && isfinite(vz))) atomicOr(vv.status, 1u);
  } else {
    vx = vv.v[i];
    vy = vv.v[V + i];
    vz = vv.v[2 * V + i];
  }
  if (do_advance) {
    px += (double)vx;
    py += (double)vy;
    pz += (double)vz;
    vv.x[i] = px;
    vv.x[V + i] = py;
    vv.x[2 * V + i] = pz;
  }
  const double P[3] = {px, py, pz};
  const int dims[3] = {L.nx, L.ny, L.nz};
  int q[3];
  bool inside = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    long long qi = hcpos::nearest(P[a]);  // floor(P + 0.5), exactly
    if (qi < 0 || qi >= dims[a]) {
      if (L.per[a]) {
        long long mm = qi % dims[a];
        qi = mm < 0 ? mm + dims[a] : mm;
      } else {
        inside = false;
      }
    }
    q[a] = (int)qi;
  }
  if (!inside) {
    vv.vnode[i] = -1;
    vv.vtile[i] = -1;
    return;
  }
  const long long nd = (long long)q[0] + (long long)L.nx * ((long long)q[1] + (long long)L.ny * q[2]);
  vv.vnode[i] = (int)nd;
  vv.vtile[i] = q[0] / tg.tx + tg.ntx * (q[1] / tg.ty + tg.nty * (q[2] / tg.tz));
  if (do_advance && L.flag[nd] != 0) {
    vv.alive[cell] = 0;
    atomicOr(vv.status, 2u);
  }
  pdl_trigger();
}

template <typename T>
cudaError_t launch_interp_advance(const LbmView<T>& L, const VertexView<T>& vv, const TileGrid& tg, int do_interp,
                                  int do_advance, int bs, cudaStream_t s) {
  if (bs <= 0) bs = 128;
  const int n = vv.nvert > 0 ? vv.nvert : 1;  // one thread at least: it advances the stamp
  return launch_kernel(k_interp_advance<T>, dim3((n + bs - 1) / bs), dim3(bs), 0, s, L.pdl, L, vv, tg, do_interp,
                       do_advance);
}

// ---------------------------------------------------------------------------
// K4: constitutive models, one CTA per cell (grid-stride over the cell list).
// Saturation constants: config/constant_defaults.h:157-173.
constexpr double kMaxVol = 0.01, kMaxArea = 0.09, kMaxBend = 0.0555, kMaxPltBend = 2.467, kMaxLink = 9.0;
constexpr double kForceLimit = 50.0;

template <typename T>
struct V3t {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3t<T> operator-(V3t<T> a, V3t<T> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ V3t<T> operator+(V3t<T> a, V3t<T> b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
__device__ __forceinline__ V3t<T> vscale(V3t<T> a, T s) {
  return {a.x * s, a.y * s, a.z * s};
}
template <typename T>
__device__ __forceinline__ V3t<T> vcross(V3t<T> a, V3t<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ T vdot(V3t<T> a, V3t<T> b) {
  T r = a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
template <typename T>
__device__ __forceinline__ T vnorm(V3t<T> a) {
  return sqrt(vdot(a, a));
}
template <typename T>
__device__ __forceinline__ V3t<T> ld3(const T* s, int k) {
  return {s[3 * k], s[3 * k + 1], s[3 * k + 2]};
}
template <typename T>
__device__ __forceinline__ void add3(T* s, int k, V3t<T> v) {
  atomicAdd(s + 3 * k, v.x);
  atomicAdd(s + 3 * k + 1, v.y);
  atomicAdd(s + 3 * k + 2, v.z);
}
// Division and normalisation: IEEE in FP64 (the plain form follows the
// reference's arithmetic), fast reciprocal / rsqrt in the FP32 mixed form.
template <typename T>
__device__ __forceinline__ T fdiv(T a, T b) {
  return a / b;
}
template <>
__device__ __forceinline__ float fdiv<float>(float a, float b) {
  return __fdividef(a, b);
}
// v / |v| with |v| returned in len (len = 0 leaves v unnormalised)
template <typename T>
__device__ __forceinline__ V3t<T> normalized(V3t<T> v, T& len) {
  len = vnorm(v);
  if (len == T(0)) return v;
  return {v.x / len, v.y / len, v.z / len};
}
template <>
__device__ __forceinline__ V3t<float> normalized<float>(V3t<float> v, float& len) {
  const float d = vdot(v, v);
  if (d == 0.f) {
    len = 0.f;
    return v;
  }
  const float inv = rsqrtf(d);
  len = d * inv;
  return {v.x * inv, v.y * inv, v.z * inv};
}
template <typename T>
__device__ __forceinline__ T third(T a) {
  return a / T(3);
}
template <>
__device__ __forceinline__ float third<float>(float a) {
  return a * (1.0f / 3.0f);
}

template <typename T>
__device__ __forceinline__ V3t<T> unit_normal(V3t<T> a, V3t<T> b, V3t<T> c) {
  V3t<T> n = vcross(b - a, c - a);
  const T l = vnorm(n);
  if (l != T(0)) return {n.x / l, n.y / l, n.z / l};
  return {T(0), T(0), T(0)};
}

template <typename T>
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double s = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

template <typename T>
__device__ __forceinline__ T rest_value(const double* d, const float* f, int k);
template <>
__device__ __forceinline__ double rest_value<double>(const double* d, const float*, int k) {
  return d[k];
}
template <>
__device__ __forceinline__ float rest_value<float>(const double*, const float* f, int k) {
  return f[k];
}

template <typename T>
size_t mechanics_smem_bytes(int nv) {
  return 34 * sizeof(double) + 6 * (size_t)nv * sizeof(T) + (size_t)nv;
}

// One CTA per cell (grid-stride over the cell list), vertex-centric: each
// thread owns vertices and sums, in a fixed order, every contribution the
// reference's face / edge / vertex loops deposit on them
// (rbcHighOrderModel.cpp:56-204, pltSimpleModel.cpp:59-205,
// wbcHighOrderModel.cpp:60-223).  Phase 1 sums the face volume terms and
// evaluates each vertex's own bending force into shared memory; after the
// block reduction of the volume, phase 2 gathers for each vertex: area and
// volume forces of its incident faces, link and membrane viscosity of its
// ring edges, the neighbours' bending reactions, the platelet dihedral terms
// of its incident and opposite edges, and its inner links.  No atomics: the
// forces are bit-reproducible.
template <typename T>
struct Face {
  V3t<T> n;  // unit normal
  T area;
  V3t<T> cen;
};

template <typename T>
__device__ __forceinline__ Face<T> face_geometry(const T* sx, const TypeDev& t, int k) {
  const int i0 = t.tris[3 * k], i1 = t.tris[3 * k + 1], i2 = t.tris[3 * k + 2];
  const V3t<T> v0 = ld3(sx, i0), v1 = ld3(sx, i1), v2 = ld3(sx, i2);
  Face<T> F;
  V3t<T> n = vcross(v1 - v0, v2 - v0);
  const T nn = vnorm(n);
  if (nn != T(0)) {
    F.area = T(0.5) * nn;
    F.n = {n.x / nn, n.y / nn, n.z / nn};
  } else {
    F.area = T(0);
    F.n = {T(0), T(0), T(0)};
  }
  F.cen = {(v0.x + v1.x + v2.x) / T(3), (v0.y + v1.y + v2.y) / T(3), (v0.z + v1.z + v2.z) / T(3)};
  return F;
}

// platelet dihedral bending force of edge e (pltSimpleModel.cpp:156-182),
// +bfv on its end points, -bfv on the two outer points
template <typename T>
__device__ __forceinline__ V3t<T> plt_bending(const T* sx, const TypeDev& t, int e) {
  const int a = t.edges[2 * e], b = t.edges[2 * e + 1];
  const V3t<T> ev = ld3(sx, b) - ld3(sx, a);
  const T L = vnorm(ev);
  const V3t<T> uv = {ev.x / L, ev.y / L, ev.z / L};
  const int* A = t.tris + 3 * t.bend_tris[2 * e];
  const int* B = t.tris + 3 * t.bend_tris[2 * e + 1];
  const V3t<T> V1 = unit_normal(ld3(sx, A[0]), ld3(sx, A[1]), ld3(sx, A[2]));
  const V3t<T> V2 = unit_normal(ld3(sx, B[0]), ld3(sx, B[1]), ld3(sx, B[2]));
  const T angle = atan2(vdot(vcross(V1, V2), uv), vdot(V1, V2));
  const T af = angle - rest_value<T>(t.edge_angle0, t.edge_angle0f, e);
  const T fm = (T)t.k_bend * (af + af / fabs(T(kMaxPltBend) - af * af));
  return vscale(V1 + V2, fm * T(0.5));
}

// spreadParticleForce of the next step for global vertex gi with the force
// just assembled (core/hemoCellParticleField.cpp:841-863): FORCE_LIMIT clamp
// (the stored force stays unclamped, as after the reference's constitutive
// model), plus the repulsion force, spread with the phi2 weights; the
// stencil nodes are tagged for the interpolation.
template <typename T>
__device__ __forceinline__ void spread_vertex(const MechView<T>& M, int gi, V3t<T> f) {
  const VertexView<T>& vv = M.vv;
  const long long V = vv.V;
  T mag = f.x * f.x;
  mag += f.y * f.y;
  mag += f.z * f.z;
  mag = sqrt(mag);
  if (mag > M.f_limit) f = vscale(f, M.f_limit / mag);
  if (vv.frep_cell) f = f + V3t<T>{vv.frep_cell[gi], vv.frep_cell[V + gi], vv.frep_cell[2 * V + gi]};
  if (vv.frep_wall) f = f + V3t<T>{vv.frep_wall[gi], vv.frep_wall[V + gi], vv.frep_wall[2 * V + gi]};
  Kern<T> K;
  ibm_weights(M.L, vv.x[gi], vv.x[V + gi], vv.x[2 * V + gi], K);
  const uint32_t stamp = *M.L.stamp + (M.fuse_advance ? 1u : 0u);
  T* F = const_cast<T*>(M.L.Fcur);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (K.node[j] < 0) continue;
    if (M.L.ntag) M.L.ntag[K.node[j]] = stamp;
    FieldLayout<T>::add(F, M.L.N, K.node[j], f.x * K.w[j], f.y * K.w[j], f.z * K.w[j]);
  }
}

// Interpolation and advance of one cell's vertices by the CTA that then
// assembles its forces (the step's interpolate + advance stage fused in front
// of the constitutive model): velocity from the node velocities with the
// phi2 weights, Euler step, nearest node and tile, and the cell's deletion
// when a vertex reaches a wall node (core/hemoCellParticleField.cpp:566-588,
// :819-839).
// voff and alive are the cell's first vertex and its state before the step;
// `hit` is a shared flag the caller cleared before its last barrier.  Returns
// whether the cell is still alive; the deletion is written to the cell's state
// by thread 0.  Ends with a barrier: every vertex is advanced and binned.
template <typename T>
__device__ __forceinline__ bool advance_cell(const MechView<T>& M, const TypeDev& t, int cell, int voff, bool alive,
                                             int& hit) {
  const VertexView<T>& vv = M.vv;
  const LbmView<T>& L = M.L;
  const long long V = vv.V;
  for (int k = threadIdx.x; k < t.nv; k += blockDim.x) {
    const int i = voff + k;
    if (!alive) {
      vv.vnode[i] = -1;
      vv.vtile[i] = -1;
      continue;
    }
    double px = vv.x[i], py = vv.x[V + i], pz = vv.x[2 * V + i];
    Kern<T> K;
    ibm_weights(L, px, py, pz, K);
    T vx = T(0), vy = T(0), vz = T(0);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      if (K.node[j] < 0) continue;
      T ux, uy, uz;
      FieldLayout<T>::load(L.unode, L.N, K.node[j], ux, uy, uz);
      vx += ux * K.w[j];
      vy += uy * K.w[j];
      vz += uz * K.w[j];
    }
    vv.v[i] = vx;
    vv.v[V + i] = vy;
    vv.v[2 * V + i] = vz;
    if (!(isfinite(vx) && isfinite(vy) && isfinite(vz))) atomicOr(vv.status, STATUS_NONFINITE);
    px += (double)vx;
    py += (double)vy;
    pz += (double)vz;
    vv.x[i] = px;
    vv.x[V + i] = py;
    vv.x[2 * V + i] = pz;
    const double P[3] = {px, py, pz};
    const int dims[3] = {L.nx, L.ny, L.nz};
    int q[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
      long long qi = hcpos::nearest(P[a]);  // floor(P + 0.5), exactly
      if (qi < 0 || qi >= dims[a]) {
        if (L.per[a]) {
          const long long mm = qi % dims[a];
          qi = mm < 0 ? mm + dims[a] : mm;
        } else {
          inside = false;
        }
      }
      q[a] = (int)qi;
    }
    if (!inside) {
      vv.vnode[i] = -1;
      vv.vtile[i] = -1;
      continue;
    }
    const long long nd = (long long)q[0] + (long long)L.nx * ((long long)q[1] + (long long)L.ny * q[2]);
    vv.vnode[i] = (int)nd;
    vv.vtile[i] = q[0] / M.tg.tx + M.tg.ntx * (q[1] / M.tg.ty + M.tg.nty * (q[2] / M.tg.tz));
    if (L.flag[nd] != 0) hit = 1;
  }
  __syncthreads();
  const bool deleted = alive && hit;
  if (threadIdx.x == 0 && deleted) {
    vv.alive[cell] = 0;
    atomicOr(vv.status, STATUS_CELL_DELETED);
  }
  return alive && !deleted;
}

// The vertex-centric force assembly of one cell (variant 0; the staged
// variant falls back to it for cell types too large for its shared memory).
// sx holds 6 nv T + nv bytes of shared memory after `red` (34 doubles).
template <typename T>
__device__ __forceinline__ void gather_cell(const MechView<T>& M, const TypeDev& t, int voff, bool alive, double* red,
                                            T* sx) {
  const VertexView<T>& vv = M.vv;
  const long long V = vv.V;
  const int tid = threadIdx.x, bs = blockDim.x;
  constexpr bool kF64 = sizeof(T) == 8;
  const int nv = t.nv;
  T* sbf = sx + 3 * nv;  // own bending force per vertex
  uint8_t* srn = reinterpret_cast<uint8_t*>(sbf + 3 * nv);  // valence per vertex
  if (!HC_IN(vv.status, (long long)voff + nv - 1, V)) return;  // the cell's vertices in the arrays
  for (int k = tid; k < nv; k += bs) srn[k] = (uint8_t)t.ring_n[k];
  // positions relative to the cell's vertex 0 (translation invariant forces;
  // the volume sum stays well conditioned far from the origin)
  const double r0x = vv.x[voff], r0y = vv.x[V + voff], r0z = vv.x[2 * V + voff];
  for (int k = tid; k < nv; k += bs) {
    sx[3 * k] = (T)(vv.x[voff + k] - r0x);
    sx[3 * k + 1] = (T)(vv.x[V + voff + k] - r0y);
    sx[3 * k + 2] = (T)(vv.x[2 * V + voff + k] - r0z);
  }
  __syncthreads();
  if (!alive) {
    for (int k = tid; k < nv; k += bs) {
      vv.f[voff + k] = T(0);
      vv.f[V + voff + k] = T(0);
      vv.f[2 * V + voff + k] = T(0);
    }
    return;
  }
  // --- phase 1: face volume terms, own bending force (rbcHighOrderModel.cpp:62-68, :127-157)
  double vol = 0.0;
  for (int k = tid; k < t.nf; k += bs) {
    const V3t<T> v0 = ld3(sx, t.tris[3 * k]), v1 = ld3(sx, t.tris[3 * k + 1]), v2 = ld3(sx, t.tris[3 * k + 2]);
    if (kF64) {
      const double v210 = (double)v2.x * v1.y * v0.z, v120 = (double)v1.x * v2.y * v0.z;
      const double v201 = (double)v2.x * v0.y * v1.z, v021 = (double)v0.x * v2.y * v1.z;
      const double v102 = (double)v1.x * v0.y * v2.z, v012 = (double)v0.x * v1.y * v2.z;
      vol += (-v210 + v120 + v201 - v021 - v102 + v012);
    } else {
      // v0 . ((v1-v0) x (v2-v0)) == v0 . (v1 x v2): FP32 term, FP64 sum
      vol += (double)vdot(v0, vcross(v1 - v0, v2 - v0));
    }
  }
  if (t.model != 1) {
    for (int i = tid; i < nv; i += bs) {
      const int rn = t.ring_n[i];
      const int* rg = t.ring + 6 * i;
      const V3t<T> xi = ld3(sx, i);
      V3t<T> sum = {T(0), T(0), T(0)};
      for (int j = 0; j < rn; ++j) sum = sum + ld3(sx, rg[j]);
      const V3t<T> mid = {fdiv(sum.x, (T)rn), fdiv(sum.y, (T)rn), fdiv(sum.z, (T)rn)};
      const V3t<T> dev = mid - xi;
      V3t<T> pn = {T(0), T(0), T(0)};
      V3t<T> a = ld3(sx, rg[0]) - xi;
      const V3t<T> first = a;
      for (int j = 0; j < rn; ++j) {
        const V3t<T> b = (j + 1 < rn) ? ld3(sx, rg[j + 1]) - xi : first;
        T l;
        pn = pn + normalized(vcross(a, b), l);
        a = b;
      }
      T pl;
      pn = normalized(pn, pl);
      const T ndev = vdot(pn, dev);
      const T dDev = fdiv(ndev - rest_value<T>(t.patch_d0, t.patch_d0f, i), (T)t.edge_mean_eq);
      const V3t<T> bf = vscale(pn, (T)t.k_bend * (dDev + fdiv(dDev, fabs(T(kMaxBend) - dDev * dDev))));
      sbf[3 * i] = bf.x;
      sbf[3 * i + 1] = bf.y;
      sbf[3 * i + 2] = bf.z;
    }
  }
  block_sum<T>(vol, red);  // red[32] = sum over the block (synchronises)
  // volume constraint in FP64 (rbcHighOrderModel.cpp:100-104), by one thread
  if (tid == 0) {
    const double volume = red[32] * (1.0 / 6.0);
    const double vfr = (volume - t.volume_eq) / t.volume_eq;
    const double vf = -t.k_volume * vfr / fabs(kMaxVol - vfr * vfr);
    red[33] = vf;
    red[31] = vf / t.area_mean_eq;
  }
  __syncthreads();
  const T vforce = (T)red[33];
  const T vforce_per_area = (T)red[31];
  const T area_mean = (T)t.area_mean_eq;
  const bool visc = (t.model != 0) || (t.eta_m != 0.0);
  // --- phase 2: gather per vertex
  for (int i = tid; i < nv; i += bs) {
    const int rn = t.ring_n[i];
    const V3t<T> xi = ld3(sx, i);
    V3t<T> f = {T(0), T(0), T(0)};
    V3t<T> vi = {T(0), T(0), T(0)};
    if (visc) vi = {vv.v[voff + i], vv.v[V + voff + i], vv.v[2 * V + voff + i]};
    int rs[6], rot[6];
    T a0s[6], l0s[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j < rn) {
        rs[j] = t.ring[6 * i + j];
        rot[j] = t.slot_rot[6 * i + j];
        a0s[j] = rest_value<T>(t.slot_a0, t.slot_a0f, 6 * i + j);
        l0s[j] = rest_value<T>(t.slot_l0, t.slot_l0f, 6 * i + j);
      }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j >= rn) break;
      const int r = rs[j];
      const int r1 = rs[j + 1 < rn ? j + 1 : 0];
      // incident face (i, r, r1) in the reference's corner order: area force
      // on this corner and the face's volume force
      const V3t<T> xr = ld3(sx, r), xr1 = ld3(sx, r1);
      const V3t<T> c0 = rot[j] == 0 ? xi : (rot[j] == 1 ? xr1 : xr);
      const V3t<T> c1 = rot[j] == 0 ? xr : (rot[j] == 1 ? xi : xr1);
      const V3t<T> c2 = rot[j] == 0 ? xr1 : (rot[j] == 1 ? xr : xi);
      Face<T> F;
      {
        T nn;
        const V3t<T> n = normalized(vcross(c1 - c0, c2 - c0), nn);
        if (nn != T(0)) {
          F.area = T(0.5) * nn;
          F.n = n;
        } else {
          F.area = T(0);
          F.n = {T(0), T(0), T(0)};
        }
        F.cen = {third(c0.x + c1.x + c2.x), third(c0.y + c1.y + c2.y), third(c0.z + c1.z + c2.z)};
      }
      const T a0 = a0s[j];
      const T ar = fdiv(F.area - a0, a0);
      const T afm = (T)t.k_area * (ar + fdiv(ar, fabs(T(kMaxArea) - ar * ar)));
      f = f + vscale(F.cen - xi, afm);
      if (kF64) f = f + vscale(vscale(F.n, vforce), F.area / area_mean);
      else f = f + vscale(F.n, vforce_per_area * F.area);
      // ring edge (i, r): link force toward r when stretched, viscosity
      const int e = t.vedge[6 * i + j];
      T L;
      const V3t<T> uv = normalized(xr - xi, L);
      const T l0 = l0s[j];
      const T ef = fdiv(L - l0, l0);
      f = f + vscale(uv, (T)t.k_link * (ef + fdiv(ef, fabs(T(kMaxLink) - ef * ef))));
      if (visc) {
        const V3t<T> vr = {vv.v[voff + r], vv.v[V + voff + r], vv.v[2 * V + voff + r]};
        V3t<T> fv = vscale(vscale(uv, vdot(vr - vi, uv)), (T)t.eta_m);
        const T mm = vnorm(fv);
        if (mm > T(kForceLimit / 4.0)) fv = vscale(fv, T(kForceLimit / 4.0) / mm);
        f = f + fv;
      }
      if (t.model != 1) {
        // neighbour's bending reaction -bf_r / n_r
        const T rnr = (T)srn[r];
        f = f + V3t<T>{fdiv(-sbf[3 * r], rnr), fdiv(-sbf[3 * r + 1], rnr), fdiv(-sbf[3 * r + 2], rnr)};
      } else {
        // platelet dihedral terms: end point of edge e, outer point of the opposite edge
        f = f + plt_bending(sx, t, e);
        f = f - plt_bending(sx, t, t.vopp[6 * i + j]);
      }
    }
    if (t.model != 1) f = f + ld3(sbf, i);
    // inner links (pltSimpleModel.cpp:188-205, wbcHighOrderModel.cpp:202-223)
    for (int q = t.vinner_off[i]; q < t.vinner_off[i + 1]; ++q) {
      const int e = t.vinner[q];
      const int o = t.inner[2 * e] == i ? t.inner[2 * e + 1] : t.inner[2 * e];
      const V3t<T> ev = ld3(sx, o) - xi;
      const T L = vnorm(ev);
      const V3t<T> uv = {ev.x / L, ev.y / L, ev.z / L};  // toward the partner
      if (t.model == 1) {
        const T l0 = rest_value<T>(t.inner_l0, t.inner_l0f, e);
        f = f + vscale(uv, (T)t.k_link * T(5) * ((L - l0) / l0));
      } else if (t.model == 2) {
        if (L < T(2) * (T)t.radius) f = f - vscale(vscale(uv, T(1) - L / (T(2) * (T)t.radius)), (T)t.k_cyto);
        if (L < T(2) * (T)t.core_radius)
          f = f - vscale(vscale(uv, T(1) - L / (T(2) * (T)t.core_radius)), (T)t.k_inner_rigid);
      }
    }
    vv.f[voff + i] = f.x;
    vv.f[V + voff + i] = f.y;
    vv.f[2 * V + voff + i] = f.z;
    if (M.fuse_spread) spread_vertex(M, voff + i, f);
  }
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 384 : 768) k_mechanics(const MechView<T> M) {
  pdl_wait();
  extern __shared__ double smem_d[];
  __shared__ TypeDev tshared;
  double* red = smem_d;  // 34 doubles
  T* sx = reinterpret_cast<T*>(smem_d + 34);
  __shared__ int hit;
  for (int ci = blockIdx.x; ci < M.ncells; ci += gridDim.x) {
    const int cell = M.cells[ci];
    __syncthreads();  // previous cell fully written out
    if (threadIdx.x == 0) {
      tshared = M.types[M.cell_type[cell]];
      hit = 0;
    }
    // the cell's scalars load while thread 0 fetches the type
    const int voff = M.cell_voff[cell];
    bool alive = M.vv.alive[cell] != 0;
    __syncthreads();
    if (M.fuse_advance) alive = advance_cell(M, tshared, cell, voff, alive, hit);
    gather_cell(M, tshared, voff, alive, red, sx);
  }
  pdl_trigger();
}

// Staged variant (2): every face's area-force scalar, centroid and
// area-weighted normal, and every edge's link force (with membrane viscosity
// and the platelet dihedral force) are computed once into shared memory;
// each vertex then gathers the terms of its incident faces and edges, its own
// and its neighbours' bending, and its inner links.  Deterministic like the
// vertex-centric variant, which computes each face and edge once per
// incident vertex; a cell type whose terms do not fit the launch's shared
// memory takes that variant's path.  Shared layout after `red` (34 doubles):
// positions 3 nv, own bending 3 nv, faces 7 nf (centroid, area-force scalar,
// area x unit normal), edges 3 ne (force on the lower-numbered end), platelet
// dihedral 3 ne (platelets only), valence nv bytes.
template <typename T>
__host__ __device__ __forceinline__ size_t staged_smem_bytes(int model, int nv, int nf, int ne) {
  const size_t words = 6 * (size_t)nv + 7 * (size_t)nf + 3 * (size_t)ne * (model == 1 ? 2 : 1);
  return 34 * sizeof(double) + words * sizeof(T) + (size_t)nv;
}

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 384 : 768) k_mechanics_staged(const MechView<T> M) {
  pdl_wait();
  extern __shared__ double smem_d[];
  __shared__ TypeDev tshared;
  double* red = smem_d;
  T* sx = reinterpret_cast<T*>(smem_d + 34);
  const VertexView<T>& vv = M.vv;
  const long long V = vv.V;
  const int tid = threadIdx.x, bs = blockDim.x;
  constexpr bool kF64 = sizeof(T) == 8;
  __shared__ int hit;
  for (int ci = blockIdx.x; ci < M.ncells; ci += gridDim.x) {
    const int cell = M.cells[ci];
    __syncthreads();
    if (tid == 0) {
      tshared = M.types[M.cell_type[cell]];
      hit = 0;
    }
    const int voff = M.cell_voff[cell];
    bool alive = vv.alive[cell] != 0;
    __syncthreads();
    const TypeDev& t = tshared;
    if (M.fuse_advance) alive = advance_cell(M, t, cell, voff, alive, hit);
    if (staged_smem_bytes<T>(t.model, t.nv, t.nf, t.ne) > (size_t)M.dyn_smem) {
      gather_cell(M, t, voff, alive, red, sx);
      continue;
    }
    const int nv = t.nv, nf = t.nf, ne = t.ne;
    const bool plt = t.model == 1;
    T* sbf = sx + 3 * nv;
    T* sface = sbf + 3 * nv;
    T* sedge = sface + 7 * nf;
    T* spltb = sedge + 3 * ne;
    uint8_t* srn = reinterpret_cast<uint8_t*>(spltb + (plt ? 3 * ne : 0));
    const double r0x = vv.x[voff], r0y = vv.x[V + voff], r0z = vv.x[2 * V + voff];
    for (int k = tid; k < nv; k += bs) {
      srn[k] = (uint8_t)t.ring_n[k];
      sx[3 * k] = (T)(vv.x[voff + k] - r0x);
      sx[3 * k + 1] = (T)(vv.x[V + voff + k] - r0y);
      sx[3 * k + 2] = (T)(vv.x[2 * V + voff + k] - r0z);
    }
    __syncthreads();
    if (!alive) {
      for (int k = tid; k < nv; k += bs) {
        vv.f[voff + k] = T(0);
        vv.f[V + voff + k] = T(0);
        vv.f[2 * V + voff + k] = T(0);
      }
      continue;
    }
    const bool visc = (t.model != 0) || (t.eta_m != 0.0);
    // --- phase A: faces, edges and bending, each once
    double vol = 0.0;
    for (int k = tid; k < nf; k += bs) {
      const V3t<T> v0 = ld3(sx, t.tris[3 * k]), v1 = ld3(sx, t.tris[3 * k + 1]), v2 = ld3(sx, t.tris[3 * k + 2]);
      const V3t<T> c = vcross(v1 - v0, v2 - v0);
      if (kF64) {
        const double v210 = (double)v2.x * v1.y * v0.z, v120 = (double)v1.x * v2.y * v0.z;
        const double v201 = (double)v2.x * v0.y * v1.z, v021 = (double)v0.x * v2.y * v1.z;
        const double v102 = (double)v1.x * v0.y * v2.z, v012 = (double)v0.x * v1.y * v2.z;
        vol += (-v210 + v120 + v201 - v021 - v102 + v012);
      } else {
        vol += (double)vdot(v0, c);
      }
      T nn;
      const V3t<T> n = normalized(c, nn);
      const T area = nn != T(0) ? T(0.5) * nn : T(0);
      const V3t<T> na = nn != T(0) ? vscale(n, area) : V3t<T>{T(0), T(0), T(0)};
      const T a0 = rest_value<T>(t.tri_a0, t.tri_a0f, k);
      const T ar = fdiv(area - a0, a0);
      T* q = sface + 7 * k;
      q[0] = third(v0.x + v1.x + v2.x);
      q[1] = third(v0.y + v1.y + v2.y);
      q[2] = third(v0.z + v1.z + v2.z);
      q[3] = (T)t.k_area * (ar + fdiv(ar, fabs(T(kMaxArea) - ar * ar)));
      q[4] = na.x;
      q[5] = na.y;
      q[6] = na.z;
    }
    for (int e = tid; e < ne; e += bs) {
      const int a = t.edges[2 * e], b = t.edges[2 * e + 1];
      T L;
      const V3t<T> uv = normalized(ld3(sx, b) - ld3(sx, a), L);
      const T l0 = rest_value<T>(t.edge_l0, t.edge_l0f, e);
      const T ef = fdiv(L - l0, l0);
      V3t<T> fe = vscale(uv, (T)t.k_link * (ef + fdiv(ef, fabs(T(kMaxLink) - ef * ef))));
      if (visc) {
        const V3t<T> va = {vv.v[voff + a], vv.v[V + voff + a], vv.v[2 * V + voff + a]};
        const V3t<T> vb = {vv.v[voff + b], vv.v[V + voff + b], vv.v[2 * V + voff + b]};
        V3t<T> fv = vscale(vscale(uv, vdot(vb - va, uv)), (T)t.eta_m);
        const T mm = vnorm(fv);
        if (mm > T(kForceLimit / 4.0)) fv = vscale(fv, T(kForceLimit / 4.0) / mm);
        fe = fe + fv;
      }
      sedge[3 * e] = fe.x;
      sedge[3 * e + 1] = fe.y;
      sedge[3 * e + 2] = fe.z;
      if (plt) {
        const V3t<T> pb = plt_bending(sx, t, e);
        spltb[3 * e] = pb.x;
        spltb[3 * e + 1] = pb.y;
        spltb[3 * e + 2] = pb.z;
      }
    }
    if (!plt) {
      for (int i = tid; i < nv; i += bs) {
        const int rn = srn[i];
        const int* rg = t.ring + 6 * i;
        const V3t<T> xi = ld3(sx, i);
        V3t<T> sum = {T(0), T(0), T(0)};
        for (int j = 0; j < rn; ++j) sum = sum + ld3(sx, rg[j]);
        const V3t<T> dev = V3t<T>{fdiv(sum.x, (T)rn), fdiv(sum.y, (T)rn), fdiv(sum.z, (T)rn)} - xi;
        V3t<T> pn = {T(0), T(0), T(0)};
        V3t<T> a = ld3(sx, rg[0]) - xi;
        const V3t<T> first = a;
        for (int j = 0; j < rn; ++j) {
          const V3t<T> b = (j + 1 < rn) ? ld3(sx, rg[j + 1]) - xi : first;
          T l;
          pn = pn + normalized(vcross(a, b), l);
          a = b;
        }
        T pl;
        pn = normalized(pn, pl);
        const T dDev = fdiv(vdot(pn, dev) - rest_value<T>(t.patch_d0, t.patch_d0f, i), (T)t.edge_mean_eq);
        const V3t<T> bf = vscale(pn, (T)t.k_bend * (dDev + fdiv(dDev, fabs(T(kMaxBend) - dDev * dDev))));
        sbf[3 * i] = bf.x;
        sbf[3 * i + 1] = bf.y;
        sbf[3 * i + 2] = bf.z;
      }
    }
    block_sum<T>(vol, red);
    if (tid == 0) {
      const double volume = red[32] * (1.0 / 6.0);
      const double vfr = (volume - t.volume_eq) / t.volume_eq;
      const double vf = -t.k_volume * vfr / fabs(kMaxVol - vfr * vfr);
      red[31] = vf / t.area_mean_eq;
    }
    __syncthreads();
    const T vforce_per_area = (T)red[31];
    // --- phase B: gather per vertex
    for (int i = tid; i < nv; i += bs) {
      const int rn = srn[i];
      const V3t<T> xi = ld3(sx, i);
      V3t<T> f = {T(0), T(0), T(0)};
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        if (j >= rn) break;
        const int r = t.ring[6 * i + j];
        const T* q = sface + 7 * t.vface[6 * i + j];
        f = f + vscale(V3t<T>{q[0], q[1], q[2]} - xi, q[3]) + vscale(V3t<T>{q[4], q[5], q[6]}, vforce_per_area);
        const int e = t.vedge[6 * i + j];
        const V3t<T> fe = ld3(sedge, e);
        f = i < r ? f + fe : f - fe;
        if (!plt) {
          const T rnr = (T)srn[r];
          f = f - V3t<T>{fdiv(sbf[3 * r], rnr), fdiv(sbf[3 * r + 1], rnr), fdiv(sbf[3 * r + 2], rnr)};
        } else {
          f = f + ld3(spltb, e) - ld3(spltb, t.vopp[6 * i + j]);
        }
      }
      if (!plt) f = f + ld3(sbf, i);
      for (int q = t.vinner_off[i]; q < t.vinner_off[i + 1]; ++q) {
        const int e = t.vinner[q];
        const int o = t.inner[2 * e] == i ? t.inner[2 * e + 1] : t.inner[2 * e];
        const V3t<T> ev = ld3(sx, o) - xi;
        const T L = vnorm(ev);
        const V3t<T> uv = {ev.x / L, ev.y / L, ev.z / L};
        if (t.model == 1) {
          const T l0 = rest_value<T>(t.inner_l0, t.inner_l0f, e);
          f = f + vscale(uv, (T)t.k_link * T(5) * ((L - l0) / l0));
        } else if (t.model == 2) {
          if (L < T(2) * (T)t.radius) f = f - vscale(vscale(uv, T(1) - L / (T(2) * (T)t.radius)), (T)t.k_cyto);
          if (L < T(2) * (T)t.core_radius)
            f = f - vscale(vscale(uv, T(1) - L / (T(2) * (T)t.core_radius)), (T)t.k_inner_rigid);
        }
      }
      vv.f[voff + i] = f.x;
      vv.f[V + voff + i] = f.y;
      vv.f[2 * V + voff + i] = f.z;
      if (M.fuse_spread) spread_vertex(M, voff + i, f);
    }
  }
  pdl_trigger();
}

// Scatter variant (selected by the tuner): one CTA per cell.  Pass A runs the faces
// (volume terms, area force); after the block reduction of the volume, pass B
// runs the volume force of every face, the bending of every vertex (RBC,
// WBC), every edge (link, membrane viscosity, platelet dihedral bending) and
// every inner link as one merged item loop.  Forces accumulate in shared
// memory and are written once.
template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 384 : 768) k_mechanics_scatter(const MechView<T> M) {
  pdl_wait();
  extern __shared__ double smem_d[];
  __shared__ TypeDev tshared;
  double* red = smem_d;  // 34 doubles
  T* sx = reinterpret_cast<T*>(smem_d + 34);
  const VertexView<T>& vv = M.vv;
  const long long V = vv.V;
  const int tid = threadIdx.x, bs = blockDim.x;
  constexpr bool kF64 = sizeof(T) == 8;
  for (int ci = blockIdx.x; ci < M.ncells; ci += gridDim.x) {
    const int cell = M.cells[ci];
    __syncthreads();  // previous cell fully written out
    if (tid == 0) tshared = M.types[M.cell_type[cell]];
    __syncthreads();
    const TypeDev& t = tshared;
    const int nv = t.nv;
    const int voff = M.cell_voff[cell];
    T* sf = sx + 3 * nv;
    const bool alive = vv.alive[cell] != 0;
    const double r0x = vv.x[voff], r0y = vv.x[V + voff], r0z = vv.x[2 * V + voff];
    for (int k = tid; k < nv; k += bs) {
      sx[3 * k] = (T)(vv.x[voff + k] - r0x);
      sx[3 * k + 1] = (T)(vv.x[V + voff + k] - r0y);
      sx[3 * k + 2] = (T)(vv.x[2 * V + voff + k] - r0z);
      sf[3 * k] = T(0);
      sf[3 * k + 1] = T(0);
      sf[3 * k + 2] = T(0);
    }
    __syncthreads();
    if (alive) {
      // --- pass A: faces, volume terms and area force (rbcHighOrderModel.cpp:56-98)
      double vol = 0.0;
      for (int k = tid; k < t.nf; k += bs) {
        const int i0 = t.tris[3 * k], i1 = t.tris[3 * k + 1], i2 = t.tris[3 * k + 2];
        const V3t<T> v0 = ld3(sx, i0), v1 = ld3(sx, i1), v2 = ld3(sx, i2);
        V3t<T> n = vcross(v1 - v0, v2 - v0);
        if (kF64) {
          const double v210 = (double)v2.x * v1.y * v0.z, v120 = (double)v1.x * v2.y * v0.z;
          const double v201 = (double)v2.x * v0.y * v1.z, v021 = (double)v0.x * v2.y * v1.z;
          const double v102 = (double)v1.x * v0.y * v2.z, v012 = (double)v0.x * v1.y * v2.z;
          vol += (-v210 + v120 + v201 - v021 - v102 + v012);
        } else {
          // v0 . ((v1-v0) x (v2-v0)) == v0 . (v1 x v2): FP32 term, FP64 sum
          vol += (double)vdot(v0, n);
        }
        const T nn = vnorm(n);
        T area;
        if (nn != T(0)) {
          area = T(0.5) * nn;
          n = {n.x / nn, n.y / nn, n.z / nn};
        } else {
          area = T(0);
        }
        const T a0 = rest_value<T>(t.tri_a0, t.tri_a0f, k);
        const T ar = (area - a0) / a0;
        const T afm = (T)t.k_area * (ar + ar / fabs(T(kMaxArea) - ar * ar));
        const V3t<T> cen = {(v0.x + v1.x + v2.x) / T(3), (v0.y + v1.y + v2.y) / T(3), (v0.z + v1.z + v2.z) / T(3)};
        add3(sf, i0, vscale(cen - v0, afm));
        add3(sf, i1, vscale(cen - v1, afm));
        add3(sf, i2, vscale(cen - v2, afm));
      }
      const double volume = block_sum<T>(vol, red) * (1.0 / 6.0);
      // volume constraint in FP64 (rbcHighOrderModel.cpp:100-104)
      const double vfr = (volume - t.volume_eq) / t.volume_eq;
      const double vforce = -t.k_volume * vfr / fabs(kMaxVol - vfr * vfr);
      const T vforce_per_area = (T)(vforce / t.area_mean_eq);
      const bool visc = (t.model != 0) || (t.eta_m != 0.0);
      const int nb = (t.model != 1) ? nv : 0;
      const int e0 = t.nf + nb, e1 = e0 + t.ne, total = e1 + t.ni;
      // --- pass B: volume force, bending, edges, inner links
      for (int k = tid; k < total; k += bs) {
        if (k < t.nf) {
          // volume force per face (rbcHighOrderModel.cpp:103-124)
          const int i0 = t.tris[3 * k], i1 = t.tris[3 * k + 1], i2 = t.tris[3 * k + 2];
          const V3t<T> v0 = ld3(sx, i0), v1 = ld3(sx, i1), v2 = ld3(sx, i2);
          V3t<T> n = vcross(v1 - v0, v2 - v0);
          const T nn = vnorm(n);
          T area;
          if (nn != T(0)) {
            area = T(0.5) * nn;
            n = {n.x / nn, n.y / nn, n.z / nn};
          } else {
            area = T(0);
            n = {T(0), T(0), T(0)};
          }
          V3t<T> lvf;
          if (kF64) lvf = vscale(vscale(n, (T)vforce), area / (T)t.area_mean_eq);
          else lvf = vscale(n, vforce_per_area * area);
          add3(sf, i0, lvf);
          add3(sf, i1, lvf);
          add3(sf, i2, lvf);
        } else if (k < e0) {
          // bending per vertex (rbcHighOrderModel.cpp:127-166)
          const int i = k - t.nf;
          const int rn = t.ring_n[i];
          const int* rg = t.ring + 6 * i;
          const V3t<T> xi = ld3(sx, i);
          V3t<T> sum = {T(0), T(0), T(0)};
          for (int j = 0; j < rn; ++j) sum = sum + ld3(sx, rg[j]);
          const V3t<T> mid = {sum.x / (T)rn, sum.y / (T)rn, sum.z / (T)rn};
          const V3t<T> dev = mid - xi;
          V3t<T> pn = {T(0), T(0), T(0)};
          V3t<T> a = ld3(sx, rg[0]) - xi;
          const V3t<T> first = a;
          for (int j = 0; j < rn; ++j) {
            const V3t<T> b = (j + 1 < rn) ? ld3(sx, rg[j + 1]) - xi : first;
            V3t<T> tn = vcross(a, b);
            const T l = vnorm(tn);
            pn = pn + V3t<T>{tn.x / l, tn.y / l, tn.z / l};
            a = b;
          }
          const T pl = vnorm(pn);
          pn = {pn.x / pl, pn.y / pl, pn.z / pl};
          const T ndev = vdot(pn, dev);
          const T dDev = (ndev - rest_value<T>(t.patch_d0, t.patch_d0f, i)) / (T)t.edge_mean_eq;
          const V3t<T> bf = vscale(pn, (T)t.k_bend * (dDev + dDev / fabs(T(kMaxBend) - dDev * dDev)));
          add3(sf, i, bf);
          const V3t<T> nbf = {-bf.x / (T)rn, -bf.y / (T)rn, -bf.z / (T)rn};
          for (int j = 0; j < rn; ++j) add3(sf, rg[j], nbf);
        } else if (k < e1) {
          // link, membrane viscosity, platelet dihedral bending
          const int e = k - e0;
          const int a = t.edges[2 * e], b = t.edges[2 * e + 1];
          const V3t<T> p0 = ld3(sx, a), p1 = ld3(sx, b);
          const V3t<T> ev = p1 - p0;
          const T L = vnorm(ev);
          const V3t<T> uv = {ev.x / L, ev.y / L, ev.z / L};
          const T l0 = rest_value<T>(t.edge_l0, t.edge_l0f, e);
          const T ef = (L - l0) / l0;
          const T fs = (T)t.k_link * (ef + ef / fabs(T(kMaxLink) - ef * ef));
          const V3t<T> force = vscale(uv, fs);
          V3t<T> fa = force, fb = {-force.x, -force.y, -force.z};
          if (visc) {
            const V3t<T> va = {vv.v[voff + a], vv.v[V + voff + a], vv.v[2 * V + voff + a]};
            const V3t<T> vb = {vv.v[voff + b], vv.v[V + voff + b], vv.v[2 * V + voff + b]};
            V3t<T> fv = vscale(vscale(uv, vdot(vb - va, uv)), (T)t.eta_m);
            const T mm = vnorm(fv);
            if (mm > T(kForceLimit / 4.0)) fv = vscale(fv, T(kForceLimit / 4.0) / mm);
            fa = fa + fv;
            fb = fb - fv;
          }
          if (t.model == 1) {  // pltSimpleModel.cpp:156-182
            const int* A = t.tris + 3 * t.bend_tris[2 * e];
            const int* B = t.tris + 3 * t.bend_tris[2 * e + 1];
            const V3t<T> V1 = unit_normal(ld3(sx, A[0]), ld3(sx, A[1]), ld3(sx, A[2]));
            const V3t<T> V2 = unit_normal(ld3(sx, B[0]), ld3(sx, B[1]), ld3(sx, B[2]));
            const T angle = atan2(vdot(vcross(V1, V2), uv), vdot(V1, V2));
            const T af = angle - rest_value<T>(t.edge_angle0, t.edge_angle0f, e);
            const T fm = (T)t.k_bend * (af + af / fabs(T(kMaxPltBend) - af * af));
            const V3t<T> bfv = vscale(V1 + V2, fm * T(0.5));
            fa = fa + bfv;
            fb = fb + bfv;
            const V3t<T> nbv = {-bfv.x, -bfv.y, -bfv.z};
            add3(sf, t.bend_outer[2 * e], nbv);
            add3(sf, t.bend_outer[2 * e + 1], nbv);
          }
          add3(sf, a, fa);
          add3(sf, b, fb);
        } else {
          // inner links
          const int e = k - e1;
          const int a = t.inner[2 * e], b = t.inner[2 * e + 1];
          const V3t<T> ev = ld3(sx, b) - ld3(sx, a);
          const T L = vnorm(ev);
          const V3t<T> uv = {ev.x / L, ev.y / L, ev.z / L};
          if (t.model == 1) {  // pltSimpleModel.cpp:188-205
            const T l0 = rest_value<T>(t.inner_l0, t.inner_l0f, e);
            const T ef = (L - l0) / l0;
            const V3t<T> force = vscale(uv, (T)t.k_link * T(5) * ef);
            add3(sf, a, force);
            add3(sf, b, V3t<T>{-force.x, -force.y, -force.z});
          } else if (t.model == 2) {  // wbcHighOrderModel.cpp:202-223
            if (L < T(2) * (T)t.radius) {
              const V3t<T> force = vscale(vscale(uv, T(1) - L / (T(2) * (T)t.radius)), (T)t.k_cyto);
              add3(sf, a, V3t<T>{-force.x, -force.y, -force.z});
              add3(sf, b, force);
            }
            if (L < T(2) * (T)t.core_radius) {
              const V3t<T> force = vscale(vscale(uv, T(1) - L / (T(2) * (T)t.core_radius)), (T)t.k_inner_rigid);
              add3(sf, a, V3t<T>{-force.x, -force.y, -force.z});
              add3(sf, b, force);
            }
          }
        }
      }
    }
    __syncthreads();
    for (int k = tid; k < nv; k += bs) {
      vv.f[voff + k] = sf[3 * k];
      vv.f[V + voff + k] = sf[3 * k + 1];
      vv.f[2 * V + voff + k] = sf[3 * k + 2];
    }
  }
}

// Raise the kernel's dynamic shared-memory limit (done when a cell type is
// added, never inside a stream capture).
template <typename T>
cudaError_t prepare_mechanics(int smem_bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_mechanics<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_mechanics_scatter<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_mechanics_staged<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
}

size_t mechanics_staged_bytes(int model, int nv, int nf, int ne, bool f64) {
  return f64 ? staged_smem_bytes<double>(model, nv, nf, ne) : staged_smem_bytes<float>(model, nv, nf, ne);
}

// variant 0: vertex-centric gather (deterministic), 1: face/edge scatter with
// shared-memory atomics
template <typename T>
cudaError_t launch_mechanics(const MechView<T>& M, int bs, int grid, int variant, cudaStream_t s) {
  if (M.ncells <= 0) return cudaSuccess;
  if (bs <= 0) bs = 256;
  if (bs > (sizeof(T) == 8 ? 384 : 768)) bs = sizeof(T) == 8 ? 384 : 768;
  if (grid <= 0 || grid > M.ncells) grid = M.ncells;
  if (variant == 1) return launch_kernel(k_mechanics_scatter<T>, dim3(grid), dim3(bs), M.dyn_smem, s, M.L.pdl, M);
  if (variant == 2) return launch_kernel(k_mechanics_staged<T>, dim3(grid), dim3(bs), M.dyn_smem, s, M.L.pdl, M);
  return launch_kernel(k_mechanics<T>, dim3(grid), dim3(bs), M.dyn_smem, s, M.L.pdl, M);
}

// device [3][Vcap] (T) -> [V][3] double
template <typename T>
__global__ void k_soa_to_aos(const T* src, double* dst, long long V, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[3 * (long long)i] = (double)src[i];
  dst[3 * (long long)i + 1] = (double)src[V + i];
  dst[3 * (long long)i + 2] = (double)src[2 * V + i];
}
template <typename T>
cudaError_t launch_soa_to_aos(const T* src, double* dst, long long V, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_soa_to_aos<T><<<(n + 255) / 256, 256, 0, s>>>(src, dst, V, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Per-vertex nearest node and tile from the current positions (update_pg,
// core/hemoCellParticleField.cpp:137-168): bin = floor(x+0.5) wrapped on
// periodic axes; vertices of removed cells or off a non-periodic axis get -1.
template <typename T>
__global__ void k_bin_vertices(const LbmView<T> L, const VertexView<T> vv, const TileGrid tg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= vv.nvert) return;
  const long long V = vv.V;
  const double P[3] = {vv.x[i], vv.x[V + i], vv.x[2 * V + i]};
  const int dims[3] = {L.nx, L.ny, L.nz};
  int q[3];
  bool inside = vv.alive[vv.vcell[i]] != 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    long long qi = hcpos::nearest(P[a]);  // floor(P + 0.5), exactly
    if (qi < 0 || qi >= dims[a]) {
      if (L.per[a]) {
        long long mm = qi % dims[a];
        qi = mm < 0 ? mm + dims[a] : mm;
      } else {
        inside = false;
      }
    }
    q[a] = (int)qi;
  }
  if (!inside) {
    vv.vnode[i] = -1;
    vv.vtile[i] = -1;
    return;
  }
  vv.vnode[i] = q[0] + L.nx * (q[1] + L.ny * q[2]);
  vv.vtile[i] = q[0] / tg.tx + tg.ntx * (q[1] / tg.ty + tg.nty * (q[2] / tg.tz));
}
template <typename T>
cudaError_t launch_bin_vertices(const LbmView<T>& L, const VertexView<T>& vv, const TileGrid& tg, cudaStream_t s) {
  if (vv.nvert <= 0) return cudaSuccess;
  k_bin_vertices<T><<<(vv.nvert + 255) / 256, 256, 0, s>>>(L, vv, tg);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Binning CSR: counts per tile, exclusive scan, fill, per-tile sort by vertex
// id (vertex ids grow with (cell, vertex id)), then per-tile unique cells.
__global__ void k_bin_count(const int* vtile, int nvert, int* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  const int t = vtile[i];
  if (t >= 0) atomicAdd(counts + t, 1);
}

// single-CTA exclusive scan of n ints into out[0..n]
__global__ void k_scan(const int* in, int n, int* out) {
  __shared__ int carry;
  __shared__ int warp_sums[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    int v = i < n ? in[i] : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      const int nw = blockDim.x >> 5;
      int s = lane < nw ? warp_sums[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const int incl = x + (wid > 0 ? warp_sums[wid - 1] : 0);
    if (i < n) out[i] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

__global__ void k_bin_fill(const int* vtile, int nvert, const int* offsets, int* cursor, int* tile_vertices) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvert) return;
  const int t = vtile[i];
  if (t < 0) return;
  const int pos = offsets[t] + atomicAdd(cursor + t, 1);
  tile_vertices[pos] = i;
}

// One CTA per tile: rank sort of the segment in shared memory (keys are
// unique vertex ids; a segment beyond 2048 takes a sorting network in place),
// then the number of distinct cells in the sorted segment.
__global__ void k_bin_sort(const int* offsets, int* tile_vertices, const int* vcell, int* tile_cell_counts) {
  __shared__ int buf[2048];
  __shared__ int ncell;
  const int t = blockIdx.x;
  const int b = offsets[t], e = offsets[t + 1], len = e - b;
  if (threadIdx.x == 0) ncell = 0;
  if (len <= 0) {
    if (threadIdx.x == 0) tile_cell_counts[t] = 0;
    return;
  }
  if (len <= 2048) {
    for (int k = threadIdx.x; k < len; k += blockDim.x) buf[k] = tile_vertices[b + k];
    __syncthreads();
    int out[8];
    int cnt = 0;
    for (int k = threadIdx.x; k < len; k += blockDim.x) {
      const int key = buf[k];
      int r = 0;
      for (int j = 0; j < len; ++j) r += buf[j] < key;
      out[cnt++] = r;
    }
    __syncthreads();
    cnt = 0;
    int keys[8];
    for (int k = threadIdx.x; k < len; k += blockDim.x) keys[cnt++] = buf[k];
    __syncthreads();
    cnt = 0;
    for (int k = threadIdx.x; k < len; k += blockDim.x) {
      buf[out[cnt]] = keys[cnt];
      cnt++;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < len; k += blockDim.x) tile_vertices[b + k] = buf[k];
    int local = 0;
    for (int k = threadIdx.x; k < len; k += blockDim.x)
      local += (k == 0 || vcell[buf[k]] != vcell[buf[k - 1]]) ? 1 : 0;
    atomicAdd(&ncell, local);
    __syncthreads();
    if (threadIdx.x == 0) tile_cell_counts[t] = ncell;
  } else {
    // A segment beyond the shared buffer is sorted in place in global memory
    // by the whole CTA: Batcher's bitonic network in its all-ascending form
    // (each merge starts by comparing element i with its mirror in the block
    // of size k, then halves the stride), over the length padded to a power
    // of two with +infinity.  A pair whose upper element lies in the padding
    // already holds the smaller key below, so it is skipped, and no index
    // past the segment is touched.  O(len log^2 len) / blockDim.x steps.
    int* seg = tile_vertices + b;
    int p2 = 1;
    while (p2 < len) p2 <<= 1;
    for (int k = 2; k <= p2; k <<= 1) {
      for (int j = k >> 1; j >= 1; j >>= 1) {
        // the first pass of a merge pairs i with its mirror in the k-block,
        // the later ones with i + j
        for (int q = threadIdx.x; q < p2 / 2; q += blockDim.x) {
          const int i = (q / j) * 2 * j + (q % j);       // lower element of pair q
          const int u = (j == k >> 1) ? (i | (k - 1)) - (i & (k - 1)) : i + j;
          if (u < len) {
            const int a = seg[i], c = seg[u];
            if (a > c) {
              seg[i] = c;
              seg[u] = a;
            }
          }
        }
        __syncthreads();
      }
    }
    int local = 0;
    for (int k = threadIdx.x; k < len; k += blockDim.x)
      local += (k == 0 || vcell[seg[k]] != vcell[seg[k - 1]]) ? 1 : 0;
    atomicAdd(&ncell, local);
    __syncthreads();
    if (threadIdx.x == 0) tile_cell_counts[t] = ncell;
  }
}

__global__ void k_tile_cells(const int* offsets, const int* tile_vertices, const int* vcell, int ntiles,
                             const int* tile_cell_offsets, int* tile_cells, int max_cells) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  int o = tile_cell_offsets[t];
  for (int k = offsets[t]; k < offsets[t + 1]; ++k) {
    const int c = vcell[tile_vertices[k]];
    if (k == offsets[t] || c != vcell[tile_vertices[k - 1]]) {
      if (o < max_cells) tile_cells[o] = c;
      o++;
    }
  }
}

cudaError_t launch_bin_csr(const int* vtile, int nvert, int ntiles, int* counts, int* offsets, int* cursor,
                           int* tile_vertices, const int* vcell, int* tile_cell_counts, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, sizeof(int) * ntiles, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(cursor, 0, sizeof(int) * ntiles, s)) != cudaSuccess) return e;
  if (nvert > 0) k_bin_count<<<(nvert + 255) / 256, 256, 0, s>>>(vtile, nvert, counts);
  k_scan<<<1, 1024, 0, s>>>(counts, ntiles, offsets);
  if (nvert > 0) k_bin_fill<<<(nvert + 255) / 256, 256, 0, s>>>(vtile, nvert, offsets, cursor, tile_vertices);
  k_bin_sort<<<ntiles, 256, 0, s>>>(offsets, tile_vertices, vcell, tile_cell_counts);
  return cudaGetLastError();
}

cudaError_t launch_tile_cells(const int* offsets, const int* tile_vertices, const int* vcell, int ntiles,
                              int* tile_cell_counts, int* tile_cell_offsets, int* tile_cells, int max_cells,
                              cudaStream_t s) {
  k_scan<<<1, 1024, 0, s>>>(tile_cell_counts, ntiles, tile_cell_offsets);
  k_tile_cells<<<(ntiles + 255) / 256, 256, 0, s>>>(offsets, tile_vertices, vcell, ntiles, tile_cell_offsets,
                                                    tile_cells, max_cells);
  return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(const int* in, int n, int* out, cudaStream_t s) {
  k_scan<<<1, 1024, 0, s>>>(in, n, out);
  return cudaGetLastError();
}

// Neighbour lists (the cells within the kernel halo of a tile): for tile t,
// the distinct cells with vertices in t or in one of its 26 neighbouring
// tiles (wrapped on periodic axes, cut at the others), ascending.  A 27-way
// merge of the tiles' ascending cell lists (tile_cell_offsets / tile_cells);
// `out` null counts only.
__device__ int tile_neighbour_cells(const TileGrid tg, int per_x, int per_y, int per_z, const int* tco,
                                    const int* tcells, int t, int* out) {
  const int tx = t % tg.ntx, ty = (t / tg.ntx) % tg.nty, tz = t / (tg.ntx * tg.nty);
  const int per[3] = {per_x, per_y, per_z};
  const int n3[3] = {tg.ntx, tg.nty, tg.ntz};
  int pos[27], end[27], tid[27], nl = 0;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        int c[3] = {tx + dx, ty + dy, tz + dz};
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
          if (c[a] < 0 || c[a] >= n3[a]) {
            if (per[a]) c[a] = (c[a] + n3[a]) % n3[a];
            else ok = false;
          }
        }
        if (!ok) continue;
        const int nt = c[0] + tg.ntx * (c[1] + tg.nty * c[2]);
        bool dup = false;  // a small periodic grid wraps onto the same tile
        for (int k = 0; k < nl; ++k)
          if (tid[k] == nt) dup = true;
        if (dup) continue;
        tid[nl] = nt;
        pos[nl] = tco[nt];
        end[nl] = tco[nt + 1];
        ++nl;
      }
  int count = 0, last = -1;
  for (;;) {
    int best = -1;
    for (int k = 0; k < nl; ++k)
      if (pos[k] < end[k] && (best < 0 || tcells[pos[k]] < best)) best = tcells[pos[k]];
    if (best < 0) break;
    for (int k = 0; k < nl; ++k)
      while (pos[k] < end[k] && tcells[pos[k]] == best) ++pos[k];
    if (best != last) {
      if (out) out[count] = best;
      ++count;
      last = best;
    }
  }
  return count;
}

__global__ void k_tile_neighbours(const TileGrid tg, int px, int py, int pz, const int* tco, const int* tcells,
                                  int ntiles, int* counts, const int* offsets, int* cells) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  if (offsets) tile_neighbour_cells(tg, px, py, pz, tco, tcells, t, cells + offsets[t]);
  else counts[t] = tile_neighbour_cells(tg, px, py, pz, tco, tcells, t, nullptr);
}

cudaError_t launch_tile_neighbours(const TileGrid& tg, const int per[3], const int* tile_cell_offsets,
                                   const int* tile_cells, int ntiles, int* counts, const int* offsets, int* cells,
                                   cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  k_tile_neighbours<<<(ntiles + 127) / 128, 128, 0, s>>>(tg, per[0], per[1], per[2], tile_cell_offsets, tile_cells,
                                                         ntiles, counts, offsets, cells);
  return cudaGetLastError();
}

cudaError_t launch_tile_sort(const int* offsets, int* tile_vertices, const int* vcell, int ntiles,
                             int* tile_cell_counts, cudaStream_t s) {
  k_bin_sort<<<ntiles, 256, 0, s>>>(offsets, tile_vertices, vcell, tile_cell_counts);
  return cudaGetLastError();
}

#define HC_CELL_INST(T)                                                                                        \
  template cudaError_t launch_spread<T>(const LbmView<T>&, const VertexView<T>&, double, int, cudaStream_t);   \
  template cudaError_t launch_mark_nodes<T>(const LbmView<T>&, const VertexView<T>&, cudaStream_t);            \
  template cudaError_t launch_cell_info<T>(const VertexView<T>&, const int*, const int*, const TypeDev*, int,   \
                                           double*, cudaStream_t);                                             \
  template cudaError_t launch_repulsion<T>(const LbmView<T>&, const VertexView<T>&, const RepView<T>&,          \
                                           cudaStream_t);                                                      \
  template cudaError_t launch_add_vertex_forces<T>(const VertexView<T>&, const int*, const double*, int,       \
                                                   cudaStream_t);                                              \
  template cudaError_t launch_interp_advance<T>(const LbmView<T>&, const VertexView<T>&, const TileGrid&, int, \
                                                int, int, cudaStream_t);                                       \
  template cudaError_t launch_mechanics<T>(const MechView<T>&, int, int, int, cudaStream_t);                   \
  template size_t mechanics_smem_bytes<T>(int);                                                                \
  template cudaError_t prepare_mechanics<T>(int);                                                              \
  template cudaError_t launch_soa_to_aos<T>(const T*, double*, long long, int, cudaStream_t);                  \
  template cudaError_t launch_bin_vertices<T>(const LbmView<T>&, const VertexView<T>&, const TileGrid&,         \
                                              cudaStream_t);
HC_CELL_INST(double)
HC_CELL_INST(float)

}  // namespace hcd
