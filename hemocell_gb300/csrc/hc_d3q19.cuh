// D3Q19 velocity set, force-field layout and the pull (streaming) read shared
// by the lattice and cell kernels.
//
// Population storage: f[19][N] holds the POST-COLLISION values f*_i - w_i of
// the last collision (pull scheme).  The post-stream (pre-collision)
// population of direction j at node x is pulled on the fly:
//   f_j(x) = f*_j(x - c_j)                             if x - c_j is fluid
//   f_j(x) = f*_i(x) - 6 w_i (c_i . u_wall),  i = opp(j)   otherwise
// (Ladd moving-wall bounce-back; u_wall is the velocity of the wall node
// x - c_j = x + c_i).  Every reader of the lattice state (collision,
// interpolation, readback) pulls, so the stored state never needs a
// separate streaming pass and all writes are aligned.
#pragma once
#include <cstdint>

#include "hc_dev.h"

namespace hcd {

__host__ __device__ constexpr int cxi(int i) {
  return (i == 1 || i == 4 || i == 5 || i == 6 || i == 7) ? -1
         : (i == 10 || i == 13 || i == 14 || i == 15 || i == 16) ? 1 : 0;
}
__host__ __device__ constexpr int cyi(int i) {
  return (i == 2 || i == 4 || i == 8 || i == 9 || i == 14) ? -1
         : (i == 5 || i == 11 || i == 13 || i == 17 || i == 18) ? 1 : 0;
}
__host__ __device__ constexpr int czi(int i) {
  return (i == 3 || i == 6 || i == 8 || i == 16 || i == 18) ? -1
         : (i == 7 || i == 9 || i == 12 || i == 15 || i == 17) ? 1 : 0;
}
__host__ __device__ constexpr int oppi(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }
__host__ __device__ constexpr double wi(int i) {
  return i == 0 ? 1.0 / 3.0 : ((cxi(i) * cxi(i) + cyi(i) * cyi(i) + czi(i) * czi(i)) == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// c . a for a lattice velocity c; the components are compile-time constants
// once the direction loop is unrolled, so zero components cost nothing.
template <typename T>
__device__ __forceinline__ T cdot(int cx, int cy, int cz, T x, T y, T z) {
  T r;
  if (cx != 0) {
    r = cx > 0 ? x : -x;
    if (cy != 0) r = cy > 0 ? r + y : r - y;
    if (cz != 0) r = cz > 0 ? r + z : r - z;
  } else if (cy != 0) {
    r = cy > 0 ? y : -y;
    if (cz != 0) r = cz > 0 ? r + z : r - z;
  } else {
    r = cz > 0 ? z : (cz < 0 ? -z : T(0));
  }
  return r;
}

// Population stores with an L2::evict_last cache policy (KEEP): the buffer a
// collide-stream writes is read next by the node-velocity pass and the next
// collide-stream, while the buffer it reads is dead once pulled, so the
// written lines are the ones worth keeping in the 129 MB L2.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void st_policy(float* p, float v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_policy(double* p, double v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(pol) : "memory");
}
template <bool KEEP, typename T>
__device__ __forceinline__ void st_pop(T* p, T v, uint64_t pol) {
  if constexpr (KEEP) st_policy(p, v, pol);
  else *p = v;
}

// Force-field layout: FP32 keeps one float4 (Fx, Fy, Fz, 0) per node so a
// spread contribution is a single vector atomic; FP64 keeps [3][N].
template <typename T>
struct FieldLayout;
template <>
struct FieldLayout<float> {
  static constexpr int kComps = 4;  // floats per node
  __device__ static __forceinline__ void load(const float* F, long long, long long n, float& x, float& y, float& z) {
    const float4 v = reinterpret_cast<const float4*>(F)[n];
    x = v.x;
    y = v.y;
    z = v.z;
  }
  __device__ static __forceinline__ void store(float* F, long long, long long n, float x, float y, float z) {
    reinterpret_cast<float4*>(F)[n] = make_float4(x, y, z, 0.f);
  }
  __device__ static __forceinline__ void add(float* F, long long, long long n, float x, float y, float z) {
    atomicAdd(reinterpret_cast<float4*>(F) + n, make_float4(x, y, z, 0.f));
  }
};
template <>
struct FieldLayout<double> {
  static constexpr int kComps = 3;
  __device__ static __forceinline__ void load(const double* F, long long N, long long n, double& x, double& y,
                                              double& z) {
    x = F[n];
    y = F[N + n];
    z = F[2 * N + n];
  }
  __device__ static __forceinline__ void store(double* F, long long N, long long n, double x, double y, double z) {
    F[n] = x;
    F[N + n] = y;
    F[2 * N + n] = z;
  }
  __device__ static __forceinline__ void add(double* F, long long N, long long n, double x, double y, double z) {
    atomicAdd(F + n, x);
    atomicAdd(F + N + n, y);
    atomicAdd(F + 2 * N + n, z);
  }
};

// Neighbour coordinates of (X,Y,Z), wrapped; a non-periodic axis that is
// left is always flagged as a bounce-back link in the node mask, so the
// wrapped index is then never used.
struct Nbr {
  int xm, xp, ym, yp, zm, zp;
  __device__ __forceinline__ Nbr(int X, int Y, int Z, int nx, int ny, int nz) {
    xm = X == 0 ? nx - 1 : X - 1;
    xp = X == nx - 1 ? 0 : X + 1;
    ym = Y == 0 ? ny - 1 : Y - 1;
    yp = Y == ny - 1 ? 0 : Y + 1;
    zm = Z == 0 ? nz - 1 : Z - 1;
    zp = Z == nz - 1 ? 0 : Z + 1;
  }
};

// Wall class of the bounce-back neighbour x + c_i (only needed when the
// node's neighbours belong to different wall classes).
template <typename T>
__device__ __forceinline__ uint32_t wall_class(const LbmView<T>& L, int i, int X, int Y, int Z, const Nbr& nb,
                                               uint32_t cls) {
  if (cls != NB_CLASS_MIXED) return cls;
  const bool out = (!L.per[0] && ((cxi(i) < 0 && X == 0) || (cxi(i) > 0 && X == L.nx - 1))) ||
                   (!L.per[1] && ((cyi(i) < 0 && Y == 0) || (cyi(i) > 0 && Y == L.ny - 1))) ||
                   (!L.per[2] && ((czi(i) < 0 && Z == 0) || (czi(i) > 0 && Z == L.nz - 1)));
  if (out) return 0u;
  const int ox = cxi(i) < 0 ? nb.xm : (cxi(i) > 0 ? nb.xp : X);
  const int oy = cyi(i) < 0 ? nb.ym : (cyi(i) > 0 ? nb.yp : Y);
  const int oz = czi(i) < 0 ? nb.zm : (czi(i) > 0 ? nb.zp : Z);
  const long long on = (long long)ox + (long long)L.nx * ((long long)oy + (long long)L.ny * oz);
  uint32_t c = HC_IN(L.status, on, L.N) ? L.flag[on] : 0u;
  return c < (uint32_t)MAX_WALL_CLASSES ? c : 0u;
}

// Post-stream populations f[j] (shifted by -w_j) of node (X,Y,Z) pulled from
// the post-collision state `src`; m is the node's bounce-back mask.
template <typename T>
__device__ __forceinline__ void pull(const LbmView<T>& L, const T* __restrict__ src, int X, int Y, int Z,
                                     long long n, uint32_t m, T f[19]) {
  const long long N = L.N;
  const Nbr nb(X, Y, Z, L.nx, L.ny, L.nz);
  const uint32_t cls = m >> NB_CLASS_SHIFT;
  f[0] = HC_IN(L.status, n, N) ? src[n] : T(0);
#pragma unroll
  for (int j = 1; j < 19; ++j) {
    const int i = oppi(j);  // x - c_j == x + c_i
    if (m & (1u << (i - 1))) {
      const uint32_t c = wall_class(L, i, X, Y, Z, nb, cls);
      const T cuw = T(cxi(i)) * L.uw[c][0] + T(cyi(i)) * L.uw[c][1] + T(czi(i)) * L.uw[c][2];
      f[j] = (HC_IN(L.status, i * N + n, 19 * N) ? src[i * N + n] : T(0)) - T(6.0 * wi(i)) * cuw;
    } else {
      const int sx = cxi(j) > 0 ? nb.xm : (cxi(j) < 0 ? nb.xp : X);
      const int sy = cyi(j) > 0 ? nb.ym : (cyi(j) < 0 ? nb.yp : Y);
      const int sz = czi(j) > 0 ? nb.zm : (czi(j) < 0 ? nb.zp : Z);
      const long long k = j * N + ((long long)sx + (long long)L.nx * ((long long)sy + (long long)L.ny * sz));
      f[j] = HC_IN(L.status, k, 19 * N) ? src[k] : T(0);
    }
  }
}

// True when node (X,Y,Z) with mask m can take pull_inline: its bounce-back
// neighbours share one wall class (a node bordering walls of different
// classes keeps the general pull).
template <typename T>
__device__ __forceinline__ bool pull_is_inline(const LbmView<T>&, int, int, int, uint32_t m) {
  return (m >> NB_CLASS_SHIFT) != NB_CLASS_MIXED;
}

// pull() without branches when 19 N < 2^31.  Population j comes from
// n + off[j], corrected by the lattice length on any axis where the
// neighbour x - c_j wraps around (a non-periodic axis never wraps here: a
// link leaving the lattice is a bounce-back link).  A bounce-back link reads
// the node's own opposite population instead (one load either way) and takes
// the moving-wall term of its class, so the lanes of a warp at a wall or on
// a face of the lattice do not diverge into the general pull.
// MW = false compiles out the moving-wall term (every wall class at rest:
// the term is then zero and the result the same).
template <typename T, bool MW = true>
__device__ __forceinline__ void pull_inline(const LbmView<T>& L, const T* __restrict__ src, int n, int X, int Y, int Z,
                                            uint32_t m, T f[19]) {
  const int N = (int)L.N, nx = L.nx, nxy = L.nx * L.ny;
  // index corrections for pulling from x-1 (c_x > 0) and from x+1 (c_x < 0), per axis
  const int cxm = X == 0 ? nx : 0, cxp = X == nx - 1 ? -nx : 0;
  const int cym = Y == 0 ? nxy : 0, cyp = Y == L.ny - 1 ? -nxy : 0;
  const int czm = Z == 0 ? N : 0, czp = Z == L.nz - 1 ? -N : 0;
  const uint32_t cls = (m >> NB_CLASS_SHIFT) & (MAX_WALL_CLASSES - 1);
  T ux = T(0), uy = T(0), uz = T(0);
  if constexpr (MW) {
    ux = L.uw[cls][0];
    uy = L.uw[cls][1];
    uz = L.uw[cls][2];
  }
  f[0] = HC_IN(L.status, n, N) ? __ldg(src + n) : T(0);
#pragma unroll
  for (int j = 1; j < 19; ++j) {
    const int i = oppi(j);  // x - c_j == x + c_i
    const bool bb = (m >> (i - 1)) & 1u;
    const int corr = (cxi(j) > 0 ? cxm : (cxi(j) < 0 ? cxp : 0)) + (cyi(j) > 0 ? cym : (cyi(j) < 0 ? cyp : 0)) +
                     (czi(j) > 0 ? czm : (czi(j) < 0 ? czp : 0));
    const int k = bb ? i * N + n : n + L.off[j] + corr;
    const T v = HC_IN(L.status, k, 19LL * N) ? __ldg(src + k) : T(0);
    if constexpr (MW) {
      const T cuw = T(cxi(i)) * ux + T(cyi(i)) * uy + T(czi(i)) * uz;
      f[j] = bb ? v - T(6.0 * wi(i)) * cuw : v;
    } else {
      f[j] = v;
    }
  }
}

// Pull of an interior node (NB_INTERIOR: no bounce-back link, on no
// periodic face, 19 N < 2^31): population j is fsrc[n + off[j]].
template <typename T>
__device__ __forceinline__ void pull_interior(const LbmView<T>& L, const T* __restrict__ src, int n, T f[19]) {
#pragma unroll
  for (int j = 0; j < 19; ++j) f[j] = HC_IN(L.status, n + L.off[j], 19 * L.N) ? __ldg(src + n + L.off[j]) : T(0);
}

// rhoBar = sum f, j = sum c f over the shifted populations, pair-wise
template <typename T>
__device__ __forceinline__ void moments(const T f[19], T& rhoBar, T& jx, T& jy, T& jz) {
  T d[10], p[10];
#pragma unroll
  for (int i = 1; i <= 9; ++i) {
    d[i] = f[i + 9] - f[i];
    p[i] = f[i + 9] + f[i];
  }
  rhoBar = f[0] + ((p[1] + p[2]) + (p[3] + p[4])) + ((p[5] + p[6]) + (p[7] + p[8])) + p[9];
  jx = (d[1] + d[4]) + (d[5] + d[6]) + d[7];
  jy = (d[2] + d[4]) - d[5] + (d[8] + d[9]);
  jz = (d[3] + d[6]) - d[7] + (d[8] - d[9]);
}

// Pull through shared memory for a block that holds whole x-rows
// (blockDim.x == nx): the 10 directions with c_x != 0 are loaded once,
// aligned, by the lane whose row neighbour needs them, then gathered from
// shared memory, so every population element is read from HBM at most once
// and only when the node that pulls it needs it (need_mask of each lane's
// own node: bit 0 = this node needs its populations).  `buf` holds
// 10 * blockDim.y * nx values, `msk` blockDim.y * nx words.  All threads of
// the block must call this (it synchronises twice).
__host__ __device__ constexpr int xdir_slot(int j) {
  return j == 1 ? 0 : j == 4 ? 1 : j == 5 ? 2 : j == 6 ? 3 : j == 7 ? 4 : j == 10 ? 5 : j == 13 ? 6 : j == 14 ? 7
         : j == 15 ? 8 : j == 16 ? 9 : -1;
}

template <typename T>
__device__ __forceinline__ void pull_rows(const LbmView<T>& L, const T* __restrict__ src, int X, int Y, int Z,
                                          long long n, uint32_t m, bool need, T* buf, uint32_t* msk, T f[19]) {
  const long long N = L.N;
  const int nx = L.nx;
  const int ty = threadIdx.y, rowlen = nx, slot_stride = blockDim.y * nx;
  const Nbr nb(X, Y, Z, L.nx, L.ny, L.nz);
  // own mask with the need bit folded in (bit 23, the solid bit, is set when not needed)
  msk[ty * rowlen + X] = need ? (m & ~NB_SOLID) : NB_SOLID;
  __syncthreads();
#pragma unroll
  for (int j = 1; j < 19; ++j) {
    if (cxi(j) == 0) continue;
    // destination of the value this lane loads: (X + c_x, same row)
    const int xd = cxi(j) > 0 ? nb.xp : nb.xm;
    const uint32_t md = msk[ty * rowlen + xd];
    const bool used = !(md & NB_SOLID) && !(md & (1u << (oppi(j) - 1)));
    if (used) {
      const int sy = cyi(j) > 0 ? nb.ym : (cyi(j) < 0 ? nb.yp : Y);
      const int sz = czi(j) > 0 ? nb.zm : (czi(j) < 0 ? nb.zp : Z);
      const long long k = j * N + ((long long)X + (long long)L.nx * ((long long)sy + (long long)L.ny * sz));
      buf[xdir_slot(j) * slot_stride + ty * rowlen + X] = HC_IN(L.status, k, 19 * N) ? src[k] : T(0);
    }
  }
  __syncthreads();
  if (!need) return;
  const uint32_t cls = m >> NB_CLASS_SHIFT;
  f[0] = HC_IN(L.status, n, N) ? src[n] : T(0);
#pragma unroll
  for (int j = 1; j < 19; ++j) {
    const int i = oppi(j);
    if (m & (1u << (i - 1))) {
      const uint32_t c = wall_class(L, i, X, Y, Z, nb, cls);
      const T cuw = T(cxi(i)) * L.uw[c][0] + T(cyi(i)) * L.uw[c][1] + T(czi(i)) * L.uw[c][2];
      f[j] = (HC_IN(L.status, i * N + n, 19 * N) ? src[i * N + n] : T(0)) - T(6.0 * wi(i)) * cuw;
    } else if (cxi(j) != 0) {
      const int xs = cxi(j) > 0 ? nb.xm : nb.xp;
      f[j] = buf[xdir_slot(j) * slot_stride + ty * rowlen + xs];
    } else {
      const int sy = cyi(j) > 0 ? nb.ym : (cyi(j) < 0 ? nb.yp : Y);
      const int sz = czi(j) > 0 ? nb.zm : (czi(j) < 0 ? nb.zp : Z);
      const long long k = j * N + ((long long)X + (long long)L.nx * ((long long)sy + (long long)L.ny * sz));
      f[j] = HC_IN(L.status, k, 19 * N) ? src[k] : T(0);
    }
  }
}

template <typename T>
size_t pull_rows_smem(int nx, int by) {
  return (size_t)10 * by * nx * sizeof(T) + (size_t)by * nx * sizeof(uint32_t);
}

__device__ __forceinline__ void node_xyz(long long n, int nx, int ny, int& X, int& Y, int& Z) {
  const long long plane = (long long)nx * ny;
  Z = (int)(n / plane);
  const long long r = n - (long long)Z * plane;
  Y = (int)(r / nx);
  X = (int)(r - (long long)Y * nx);
}

}  // namespace hcd
