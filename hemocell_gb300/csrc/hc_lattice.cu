// Lattice kernels of the GB300 HemoCell step (sm_103a):
//   K1 collide_stream  pull + D3Q19 Guo-forced BGK collision, aligned writes
//                      of the post-collision state; writes the next step's
//                      force field (body force), fusing the force reset.
//   node_velocity      post-stream velocity of the nodes the IBM stencils touch
//   moments / stream_out / stream_in / field conversions for readback and set-up
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "hc_async.cuh"
#include "hc_d3q19.cuh"

namespace hcd {

// Guo-forced BGK collision of one node from its pulled populations f and
// force F; writes the post-collision populations and the node's next force
// (the body force of plane Z).
template <typename T, typename Idx, bool KEEP = false>
__device__ __forceinline__ void collide_store(const LbmView<T>& L, Idx n, int Z, const T f[19], T Fx, T Fy, T Fz) {
  const Idx N = (Idx)L.N;
  if (!HC_IN(L.status, n, N) || !HC_IN(L.status, Z, L.nz)) return;
  uint64_t pol = 0;
  if constexpr (KEEP) pol = l2_policy_evict_last();
  T rhoBar, jx, jy, jz;
  moments(f, rhoBar, jx, jy, jz);
  const T rho = T(1) + rhoBar;
  const T invRho = T(1) / rho;
  const T ux = (jx + T(0.5) * Fx) * invRho;
  const T uy = (jy + T(0.5) * Fy) * invRho;
  const T uz = (jz + T(0.5) * Fz) * invRho;
  const T uu = ux * ux + uy * uy + uz * uz;
  const T uF = ux * Fx + uy * Fy + uz * Fz;
  const T om = L.omega;
  const T om1 = T(1) - om;
  const T hs = T(1) - T(0.5) * om;
  const T A = rhoBar - T(1.5) * rho * uu;  // even equilibrium part without w
  const T B = T(4.5) * rho;
  const T K = T(3) * rho * om;
  const T G = T(-3) * hs * uF;
  const T H = T(9) * hs;
  const T Lc = T(3) * hs;
  const T w1 = T(1.0 / 18.0);
  const T Aw1 = om * w1 * A, Bw1 = om * w1 * B, Gw1 = w1 * G, Hw1 = w1 * H, Kw1 = w1 * K, Lw1 = w1 * Lc;
  const T Aw2 = T(0.5) * Aw1, Bw2 = T(0.5) * Bw1, Gw2 = T(0.5) * Gw1, Hw2 = T(0.5) * Hw1, Kw2 = T(0.5) * Kw1,
          Lw2 = T(0.5) * Lw1;

  st_pop<KEEP>(L.fdst + n, om1 * f[0] + T(1.0 / 3.0) * (om * A + G), pol);
#pragma unroll
  for (int i = 1; i <= 9; ++i) {
    const int j = i + 9;  // c = c_j
    const T cu = cdot(cxi(j), cyi(j), czi(j), ux, uy, uz);
    const T cF = cdot(cxi(j), cyi(j), czi(j), Fx, Fy, Fz);
    const bool axis = (wi(j) > 1.0 / 20.0);
    const T Aw = axis ? Aw1 : Aw2, Bw = axis ? Bw1 : Bw2, Gw = axis ? Gw1 : Gw2;
    const T Hw = axis ? Hw1 : Hw2, Kw = axis ? Kw1 : Kw2, Lw = axis ? Lw1 : Lw2;
    const T P = (Bw * (cu * cu) + Aw) + (Hw * (cu * cF) + Gw);
    const T Q = Kw * cu + Lw * cF;
    st_pop<KEEP>(L.fdst + j * N + n, om1 * f[j] + (P + Q), pol);
    st_pop<KEEP>(L.fdst + i * N + n, om1 * f[i] + (P - Q), pol);
  }
  FieldLayout<T>::store(L.Fnext, N, n, L.bodyz[Z], L.bodyz[L.nz + Z], L.bodyz[2 * L.nz + Z]);
}

// ---------------------------------------------------------------------------
// K1.  One thread per node; blocks (bx, by) over x,y and one z-plane per
// blockIdx.z.  The collision is written per opposite pair (i, i+9), sharing
// the even and odd parts of equilibrium and Guo source:
//   f*_{+c} = (1-w) f_{+c} + P + Q,   f*_{-c} = (1-w) f_{-c} + P - Q
// with rho u = sum c f + F/2 (Guo, Zheng & Shi 2002).
// ROWS: the block spans whole x-rows and pulls through shared memory
// (pull_rows); otherwise each thread pulls directly from global memory.
// The sweep direction alternates every step (L.reverse): a pass then starts
// on the planes the previous pass wrote last, which are still in L2.
// V (direct pull with I32 only): bit 0 interior nodes take pull_interior,
// bit 1 evict-last population stores, bit 2 moving walls (clear: every wall
// class is at rest and pull_inline drops the moving-wall term).
template <typename T, bool ROWS, bool I32, int V = 4>
__global__ void __launch_bounds__(256) k_collide_stream(const LbmView<T> L) {
  pdl_wait();
  if (L.bump_stamp && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    *L.stamp += 1;
  // I32: every population index fits 32 bits (19 N < 2^31), so interior
  // nodes pull through L.off and all index arithmetic stays 32-bit
  using Idx = typename std::conditional<I32, int, long long>::type;
  extern __shared__ double k1_smem[];
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = L.reverse ? L.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
  const Idx N = (Idx)L.N;
  T f[19];
  Idx n;
  uint32_t m;
  if (ROWS) {
    const bool inside = Y < L.ny;
    n = (long long)X + (long long)L.nx * ((long long)(inside ? Y : 0) + (long long)L.ny * Z);
    m = inside ? __ldg(L.nbmask + n) : NB_SOLID;
    const bool need = !(m & NB_SOLID);
    T* buf = reinterpret_cast<T*>(k1_smem);
    uint32_t* msk = reinterpret_cast<uint32_t*>(buf + 10 * blockDim.y * L.nx);
    pull_rows(L, L.fsrc, X, inside ? Y : 0, Z, n, m, need, buf, msk, f);
    if (!need) return;
  } else {
    if (X >= L.nx || Y >= L.ny) return;
    n = (Idx)X + (Idx)L.nx * ((Idx)Y + (Idx)L.ny * Z);
    m = __ldg(L.nbmask + n);
    if (m & NB_SOLID) return;
    if (I32 && (V & 1) && (m & NB_INTERIOR)) pull_interior(L, L.fsrc, (int)n, f);
    else if (I32 && pull_is_inline(L, X, Y, Z, m)) pull_inline<T, (V & 4) != 0>(L, L.fsrc, (int)n, X, Y, Z, m, f);
    else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  }
  T Fx, Fy, Fz;
  FieldLayout<T>::load(L.Fcur, N, n, Fx, Fy, Fz);
  collide_store<T, Idx, (V & 2) != 0>(L, n, Z, f, Fx, Fy, Fz);
  pdl_trigger();
}

// ---------------------------------------------------------------------------
// K1 over the fluid nodes only.  Thread t takes the t-th fluid node in
// lattice order (from the end when L.reverse), so no lane of a warp idles on
// a wall node, as lanes of the (x, y)-block kernel do around a cylinder; runs
// of consecutive fluid nodes keep the pulls coalesced.  Needs L.fluid, which
// exists only when every index fits 32 bits.
__device__ __forceinline__ void unpack_node(uint32_t c, int& X, int& Y, int& Z) {
  X = (int)(c & 1023u);
  Y = (int)((c >> 10) & 1023u);
  Z = (int)(c >> 20);
}

// V as for k_collide_stream (bit 0 interior pull, bit 1 evict-last stores,
// bit 2 moving walls).
template <typename T, int V>
__global__ void __launch_bounds__(256) k_collide_stream_fluid(const LbmView<T> L) {
  pdl_wait();
  if (L.bump_stamp && blockIdx.x == 0 && threadIdx.x == 0) *L.stamp += 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L.nfluid) return;
  int X, Y, Z;
  unpack_node(__ldg(L.fluid + (L.reverse ? L.nfluid - 1 - t : t)), X, Y, Z);
  const int n = X + L.nx * (Y + L.ny * Z);
  const uint32_t m = __ldg(L.nbmask + n);
  T f[19];
  if ((V & 1) && (m & NB_INTERIOR)) pull_interior(L, L.fsrc, n, f);
  else if (pull_is_inline(L, X, Y, Z, m)) pull_inline<T, (V & 4) != 0>(L, L.fsrc, n, X, Y, Z, m, f);
  else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  T Fx, Fy, Fz;
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  collide_store<T, int, (V & 2) != 0>(L, n, Z, f, Fx, Fy, Fz);
  pdl_trigger();
}

template <typename T>
cudaError_t launch_collide_stream_fluid(const LbmView<T>& L, int bs, cudaStream_t s) {
  if (L.nfluid <= 0) return cudaSuccess;
  if (bs <= 0 || bs > 256) bs = 256;
  const dim3 g((L.nfluid + bs - 1) / bs), b(bs);
  switch ((L.k1var & 3) | (L.moving_walls ? 4 : 0)) {
    case 0: return launch_kernel(k_collide_stream_fluid<T, 0>, g, b, 0, s, L.pdl, L);
    case 1: return launch_kernel(k_collide_stream_fluid<T, 1>, g, b, 0, s, L.pdl, L);
    case 2: return launch_kernel(k_collide_stream_fluid<T, 2>, g, b, 0, s, L.pdl, L);
    case 3: return launch_kernel(k_collide_stream_fluid<T, 3>, g, b, 0, s, L.pdl, L);
    case 5: return launch_kernel(k_collide_stream_fluid<T, 5>, g, b, 0, s, L.pdl, L);
    case 6: return launch_kernel(k_collide_stream_fluid<T, 6>, g, b, 0, s, L.pdl, L);
    case 7: return launch_kernel(k_collide_stream_fluid<T, 7>, g, b, 0, s, L.pdl, L);
    default: return launch_kernel(k_collide_stream_fluid<T, 4>, g, b, 0, s, L.pdl, L);
  }
}

// ---------------------------------------------------------------------------
// K1 with bulk copies.  A persistent CTA owns a slab of R whole x-rows
// (y in [y0, y0+R)) and sweeps a chunk of z-planes.  For plane z, direction j
// pulls from rows y - cy_j of plane z - cz_j of population array j: one
// contiguous block of R rows (two when the slab touches the y edge and the
// rows wrap), fetched whole by cp.async.bulk into a shared-memory stage
// together with the plane's force and mask rows.  The x-shift -cx_j is then
// read from the staged row, wrapping inside it.  One thread keeps `stages`
// planes in flight; every thread computes one node of the slab from shared
// memory and writes the post-collision populations as K1 does.  Bounce-back
// links read the node's own opposite population from global memory.
template <typename T>
__device__ __forceinline__ T bounce_value(const LbmView<T>& L, int i, int X, int Y, int Z, long long n, uint32_t m) {
  const Nbr nb(X, Y, Z, L.nx, L.ny, L.nz);
  const uint32_t c = wall_class(L, i, X, Y, Z, nb, m >> NB_CLASS_SHIFT);
  const T cuw = T(cxi(i)) * L.uw[c][0] + T(cyi(i)) * L.uw[c][1] + T(czi(i)) * L.uw[c][2];
  return L.fsrc[i * L.N + n] - T(6.0 * wi(i)) * cuw;
}

template <typename T>
struct StageLayout {
  int RN;
  __device__ __host__ size_t pops() const { return 0; }
  __device__ __host__ size_t force() const { return (size_t)19 * RN * sizeof(T); }
  __device__ __host__ size_t mask() const { return force() + (size_t)RN * (sizeof(T) == 4 ? 16 : 24); }
  __device__ __host__ size_t bytes() const { return mask() + (size_t)RN * 4; }
};

template <typename T>
__global__ void __launch_bounds__(256) k_collide_stream_bulk(const LbmView<T> L, const BulkPlan P) {
  if (L.bump_stamp && blockIdx.x == 0 && threadIdx.x == 0) *L.stamp += 1;
  extern __shared__ __align__(128) unsigned char k1b_smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(k1b_smem);
  unsigned char* stage0 = k1b_smem + 128;
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  const int RN = P.R * nx;
  const StageLayout<T> SL{RN};
  const int tid = threadIdx.x;
  const int slab = blockIdx.x % P.nslab;
  const int zb = (blockIdx.x / P.nslab) * P.zlen;
  const int y0 = slab * P.R;
  const int zcount = min(P.zlen, nz - zb);
  if (zcount <= 0) return;
  const long long N = L.N;
  if (tid == 0) {
    for (int s = 0; s < P.stages; ++s) mbar_init(&bars[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto plane_of = [&](int k) { return L.reverse ? zb + zcount - 1 - k : zb + k; };
  // thread 0: fill the stage of plane k
  auto issue = [&](int k) {
    const int s = k % P.stages;
    unsigned char* st = stage0 + (size_t)s * P.stage_bytes;
    const int z = plane_of(k);
    mbar_expect_tx(&bars[s], (uint32_t)P.tx_bytes);
    const uint32_t rowb = (uint32_t)(nx * sizeof(T));
#pragma unroll 1
    for (int j = 0; j < 19; ++j) {
      int zs = z - czi(j);
      zs = zs < 0 ? zs + nz : (zs >= nz ? zs - nz : zs);
      const int ys = y0 - cyi(j);
      T* dst = reinterpret_cast<T*>(st + SL.pops()) + (size_t)j * RN;
      const T* base = L.fsrc + (long long)j * N + (long long)zs * ny * nx;
      if (ys >= 0 && ys + P.R <= ny) {
        bulk_g2s(dst, base + (long long)ys * nx, (uint32_t)P.R * rowb, &bars[s]);
      } else if (ys < 0) {  // the slab's first row comes from the last row
        bulk_g2s(dst, base + (long long)(ny - 1) * nx, rowb, &bars[s]);
        if (P.R > 1) bulk_g2s(dst + nx, base, (uint32_t)(P.R - 1) * rowb, &bars[s]);
      } else {  // the slab's last row comes from the first row
        if (P.R > 1) bulk_g2s(dst, base + (long long)ys * nx, (uint32_t)(P.R - 1) * rowb, &bars[s]);
        bulk_g2s(dst + (size_t)(P.R - 1) * nx, base, rowb, &bars[s]);
      }
    }
    const long long off = ((long long)z * ny + y0) * nx;
    if (sizeof(T) == 4) {
      bulk_g2s(st + SL.force(), reinterpret_cast<const float4*>(L.Fcur) + off, (uint32_t)RN * 16u, &bars[s]);
    } else {
      for (int a = 0; a < 3; ++a)
        bulk_g2s(st + SL.force() + (size_t)a * RN * 8, L.Fcur + a * N + off, (uint32_t)RN * 8u, &bars[s]);
    }
    bulk_g2s(st + SL.mask(), L.nbmask + off, (uint32_t)RN * 4u, &bars[s]);
  };
  int issued = 0;
  if (tid == 0)
    for (; issued < min(P.stages, zcount); ++issued) issue(issued);
  const int r = tid / nx, X = tid - r * nx, Y = y0 + r;
  int k = 0;
  bool failed = false;
  for (; k < zcount; ++k) {
    const int s = k % P.stages;
    const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((k / P.stages) & 1), P.spin_limit);
    const unsigned char* st = stage0 + (size_t)s * P.stage_bytes;
    const uint32_t m = reinterpret_cast<const uint32_t*>(st + SL.mask())[tid];
    const int Z = plane_of(k);
    if (ok && !(m & NB_SOLID)) {
      const T* sp = reinterpret_cast<const T*>(st + SL.pops());
      const long long n = (long long)X + (long long)nx * ((long long)Y + (long long)ny * Z);
      T f[19];
      f[0] = sp[tid];
#pragma unroll
      for (int j = 1; j < 19; ++j) {
        const int i = oppi(j);
        if (m & (1u << (i - 1))) {
          f[j] = bounce_value(L, i, X, Y, Z, n, m);
        } else {
          int xs = X - cxi(j);
          xs = xs < 0 ? xs + nx : (xs >= nx ? xs - nx : xs);
          f[j] = sp[j * RN + r * nx + xs];
        }
      }
      T Fx, Fy, Fz;
      if (sizeof(T) == 4) {
        const float4 v = reinterpret_cast<const float4*>(st + SL.force())[tid];
        Fx = (T)v.x;
        Fy = (T)v.y;
        Fz = (T)v.z;
      } else {
        const T* fp = reinterpret_cast<const T*>(st + SL.force());
        Fx = fp[tid];
        Fy = fp[RN + tid];
        Fz = fp[2 * RN + tid];
      }
      collide_store<T, long long>(L, n, Z, f, Fx, Fy, Fz);
    }
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (tid == 0 && issued < zcount) issue(issued++);
  }
  if (failed && tid == 0) {
    atomicOr(L.status, STATUS_WAIT_TIMEOUT);
    // let the copies already issued land before the CTA's shared memory is
    // released: each stage gets four more bounded waits.  A copy that has not
    // landed even then leaves the handle unusable; STATUS_WAIT_TIMEOUT tells
    // the host to discard it.
    for (int q = k; q < issued; ++q) {
      bool landed = false;
      for (int tries = 0; tries < 4 && !landed; ++tries)
        landed = mbar_wait_bounded(&bars[q % P.stages], (uint32_t)((q / P.stages) & 1), P.spin_limit);
      if (!landed) break;
    }
  }
}

template <typename T>
bool make_bulk_plan(int nx, int ny, int nz, int stages, int ctas_target, BulkPlan* P) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || stages < 2 || ctas_target < 1) return false;
  // cp.async.bulk wants 16-byte sizes and addresses: rows of populations and
  // forces (nx T) and of the 32-bit node mask (nx words, so nx % 4 == 0; an
  // FP64 lattice with nx = 2 mod 4 passes the first test but not this one)
  if ((nx * sizeof(T)) % 16 != 0 || (nx * sizeof(uint32_t)) % 16 != 0 || nx > 256) return false;
  int R = 0;
  for (int r = 256 / nx; r >= 1; --r)
    if (ny % r == 0) {
      R = r;
      break;
    }
  if (R == 0) return false;
  const int RN = R * nx;
  StageLayout<T> SL{RN};
  P->R = R;
  P->nslab = ny / R;
  P->stages = stages;
  P->stage_bytes = (int)((SL.bytes() + 127) / 128 * 128);
  P->tx_bytes = (int)SL.bytes();
  if (128 + (size_t)stages * P->stage_bytes > 227 * 1024) return false;
  const int zch = std::max(1, std::min(nz, (ctas_target + P->nslab - 1) / P->nslab));
  P->zlen = (nz + zch - 1) / zch;
  P->zchunks = (nz + P->zlen - 1) / P->zlen;
  P->spin_limit = 2000000000LL;
  return true;
}

template <typename T>
size_t bulk_smem_bytes(const BulkPlan& P) {
  return 128 + (size_t)P.stages * P.stage_bytes;
}

// The attribute is device-wide state shared by every handle: raise it to the
// opt-in maximum once rather than to one plan's size, which a later handle
// with a smaller plan would lower beneath this one's.
template <typename T>
cudaError_t prepare_collide_bulk(const BulkPlan& P) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if ((int)bulk_smem_bytes<T>(P) > optin) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(k_collide_stream_bulk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <typename T>
cudaError_t launch_collide_stream_bulk(const LbmView<T>& L, const BulkPlan& P, cudaStream_t s) {
  k_collide_stream_bulk<T><<<P.nslab * P.zchunks, P.R * L.nx, bulk_smem_bytes<T>(P), s>>>(L, P);
  return cudaGetLastError();
}

// bx == 0 selects the row-staged kernel with blocks of (nx, by) when nx
// allows it (nx * by <= 256); otherwise (bx, by) blocks pull directly.
template <typename T>
cudaError_t launch_collide_stream(const LbmView<T>& L, int bx, int by, cudaStream_t s) {
  if (by <= 0) by = 4;
  if (bx == 0 && L.nx <= 256) {
    while (L.nx * by > 256 && by > 1) by /= 2;
    dim3 block(L.nx, by, 1);
    dim3 grid(1, (L.ny + by - 1) / by, L.nz);
    k_collide_stream<T, true, false><<<grid, block, pull_rows_smem<T>(L.nx, by), s>>>(L);
    return cudaGetLastError();
  }
  if (bx <= 0) bx = 64;
  dim3 block(bx, by, 1);
  dim3 grid((L.nx + bx - 1) / bx, (L.ny + by - 1) / by, L.nz);
  if (L.fast) {
    switch ((L.k1var & 3) | (L.moving_walls ? 4 : 0)) {
      case 0: return launch_kernel(k_collide_stream<T, false, true, 0>, grid, block, 0, s, L.pdl, L);
      case 1: return launch_kernel(k_collide_stream<T, false, true, 1>, grid, block, 0, s, L.pdl, L);
      case 2: return launch_kernel(k_collide_stream<T, false, true, 2>, grid, block, 0, s, L.pdl, L);
      case 3: return launch_kernel(k_collide_stream<T, false, true, 3>, grid, block, 0, s, L.pdl, L);
      case 5: return launch_kernel(k_collide_stream<T, false, true, 5>, grid, block, 0, s, L.pdl, L);
      case 6: return launch_kernel(k_collide_stream<T, false, true, 6>, grid, block, 0, s, L.pdl, L);
      case 7: return launch_kernel(k_collide_stream<T, false, true, 7>, grid, block, 0, s, L.pdl, L);
      default: return launch_kernel(k_collide_stream<T, false, true, 4>, grid, block, 0, s, L.pdl, L);
    }
  }
  return launch_kernel(k_collide_stream<T, false, false>, grid, block, 0, s, L.pdl, L);
}

// ---------------------------------------------------------------------------
// Velocity u = (sum c f + F/2)/rho of the post-stream state at every node
// tagged by this step's stencils (Palabos computeVelocity for Guo forcing,
// core/hemoCellParticleField.cpp:833); L.fsrc is the post-collision state,
// L.Fcur the force of that collision.
template <typename T, bool I32>
__global__ void __launch_bounds__(256) k_node_velocity(const LbmView<T> L) {
  pdl_wait();
  using Idx = typename std::conditional<I32, int, long long>::type;
  const Idx g = (Idx)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (Idx)L.N) return;
  const Idx n = L.reverse ? (Idx)L.N - 1 - g : g;
  if (L.ntag[n] != *L.stamp) return;
  const uint32_t m = L.nbmask[n];
  int X, Y, Z;
  node_xyz((long long)n, L.nx, L.ny, X, Y, Z);
  T f[19];
  if (I32 && pull_is_inline(L, X, Y, Z, m)) pull_inline(L, L.fsrc, (int)n, X, Y, Z, m, f);
  else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  T rhoBar, jx, jy, jz, Fx, Fy, Fz;
  moments(f, rhoBar, jx, jy, jz);
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  const T rho = T(1) + rhoBar;
  FieldLayout<T>::store(L.unode, L.N, n, (jx + T(0.5) * Fx) / rho, (jy + T(0.5) * Fy) / rho,
                        (jz + T(0.5) * Fz) / rho);
  pdl_trigger();
}
template <typename T>
__global__ void __launch_bounds__(256) k_node_velocity_fluid(const LbmView<T> L) {
  pdl_wait();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= L.nfluid) return;
  int X, Y, Z;
  unpack_node(__ldg(L.fluid + (L.reverse ? L.nfluid - 1 - t : t)), X, Y, Z);
  const int n = X + L.nx * (Y + L.ny * Z);
  if (L.ntag[n] != *L.stamp) return;
  const uint32_t m = L.nbmask[n];
  T f[19];
  if (pull_is_inline(L, X, Y, Z, m)) pull_inline(L, L.fsrc, n, X, Y, Z, m, f);
  else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  T rhoBar, jx, jy, jz, Fx, Fy, Fz;
  moments(f, rhoBar, jx, jy, jz);
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  const T rho = T(1) + rhoBar;
  FieldLayout<T>::store(L.unode, L.N, n, (jx + T(0.5) * Fx) / rho, (jy + T(0.5) * Fy) / rho,
                        (jz + T(0.5) * Fz) / rho);
  pdl_trigger();
}

// Node velocity with the tagged nodes packed into whole warps.  A warp scans
// a chunk of 256 consecutive nodes (8 per lane), gathers the tagged ones in
// ascending order into shared memory and then pulls them 32 at a time, so
// the pull runs with every lane busy whatever the density of tags, and the
// scan costs one thread per 8 nodes.  Needs 19 N < 2^31 (L.fast).
template <typename T>
__device__ __forceinline__ void node_velocity_at(const LbmView<T>& L, int n) {
  const int nxy = L.nx * L.ny;
  const int Z = n / nxy, r = n - Z * nxy, Y = r / L.nx, X = r - Y * L.nx;
  const uint32_t m = L.nbmask[n];
  T f[19];
  if (pull_is_inline(L, X, Y, Z, m)) pull_inline(L, L.fsrc, n, X, Y, Z, m, f);
  else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  T rhoBar, jx, jy, jz, Fx, Fy, Fz;
  moments(f, rhoBar, jx, jy, jz);
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  const T rho = T(1) + rhoBar;
  FieldLayout<T>::store(L.unode, L.N, n, (jx + T(0.5) * Fx) / rho, (jy + T(0.5) * Fy) / rho,
                        (jz + T(0.5) * Fz) / rho);
}

template <typename T>
__global__ void __launch_bounds__(256) k_node_velocity_packed(const LbmView<T> L) {
  pdl_wait();
  __shared__ int list[8][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = (int)L.N;
  const int nchunks = (N + 255) / 256;
  const int chunk = blockIdx.x * 8 + w;
  if (chunk >= nchunks) return;
  const int c = L.reverse ? nchunks - 1 - chunk : chunk;
  const uint32_t stamp = *L.stamp;
  const int base = c * 256 + lane * 8;
  uint32_t bits = 0;
  if (base + 8 <= N) {
    const uint4 a = *reinterpret_cast<const uint4*>(L.ntag + base);
    const uint4 b = *reinterpret_cast<const uint4*>(L.ntag + base + 4);
    bits = (a.x == stamp) | (a.y == stamp) << 1 | (a.z == stamp) << 2 | (a.w == stamp) << 3 | (b.x == stamp) << 4 |
           (b.y == stamp) << 5 | (b.z == stamp) << 6 | (b.w == stamp) << 7;
  } else {
    for (int k = 0; k < 8; ++k)
      if (base + k < N && L.ntag[base + k] == stamp) bits |= 1u << k;
  }
  const int cnt = __popc(bits);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  int pos = incl - cnt;
  for (int k = 0; k < 8; ++k)
    if ((bits >> k) & 1u) list[w][pos++] = base + k;
  __syncwarp();
  for (int r = lane; r < total; r += 32) node_velocity_at(L, list[w][r]);
  pdl_trigger();
}

// Node velocity at every fluid node, in the collide-stream's (x, y)-block
// layout: whole warps of coalesced pulls, where the tagged forms pull only
// the stencil nodes through partly used sectors.  Interpolation reads only
// tagged nodes, whose values are the tagged forms' bits.  Needs 19 N < 2^31.
// INTERIOR: interior nodes take pull_interior, as the collide-stream does
// with tune[7] bit 12.  Without it every node takes pull_inline: a warp that
// holds both kinds of node (every warp of a lattice with walls across its
// rows) then issues one sequence of 19 loads instead of both.
template <typename T, bool MW, bool INTERIOR>
__global__ void __launch_bounds__(256) k_node_velocity_dense(const LbmView<T> L) {
  pdl_wait();
  const int X = blockIdx.x * blockDim.x + threadIdx.x;
  const int Y = blockIdx.y * blockDim.y + threadIdx.y;
  const int Z = L.reverse ? L.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
  if (X >= L.nx || Y >= L.ny) return;
  const int n = X + L.nx * (Y + L.ny * Z);
  const uint32_t m = __ldg(L.nbmask + n);
  if (m & NB_SOLID) return;
  T f[19];
  if (INTERIOR && (m & NB_INTERIOR)) pull_interior(L, L.fsrc, n, f);
  else if (pull_is_inline(L, X, Y, Z, m)) pull_inline<T, MW>(L, L.fsrc, n, X, Y, Z, m, f);
  else pull(L, L.fsrc, X, Y, Z, (long long)n, m, f);
  T rhoBar, jx, jy, jz, Fx, Fy, Fz;
  moments(f, rhoBar, jx, jy, jz);
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  const T rho = T(1) + rhoBar;
  FieldLayout<T>::store(L.unode, L.N, n, (jx + T(0.5) * Fx) / rho, (jy + T(0.5) * Fy) / rho,
                        (jz + T(0.5) * Fz) / rho);
  pdl_trigger();
}

template <typename T>
cudaError_t launch_node_velocity_dense(const LbmView<T>& L, cudaStream_t s) {
  const dim3 b(32, 8), g((L.nx + 31) / 32, (L.ny + 7) / 8, L.nz);
  switch ((L.k1var & 1) | (L.moving_walls ? 2 : 0)) {
    case 0: return launch_kernel(k_node_velocity_dense<T, false, false>, g, b, 0, s, L.pdl, L);
    case 1: return launch_kernel(k_node_velocity_dense<T, false, true>, g, b, 0, s, L.pdl, L);
    case 2: return launch_kernel(k_node_velocity_dense<T, true, false>, g, b, 0, s, L.pdl, L);
    default: return launch_kernel(k_node_velocity_dense<T, true, true>, g, b, 0, s, L.pdl, L);
  }
}

template <typename T>
cudaError_t launch_node_velocity_packed(const LbmView<T>& L, cudaStream_t s) {
  const long long nchunks = (L.N + 255) / 256;
  return launch_kernel(k_node_velocity_packed<T>, dim3((unsigned)((nchunks + 7) / 8)), dim3(256), 0, s, L.pdl, L);
}

template <typename T>
cudaError_t launch_node_velocity_fluid(const LbmView<T>& L, cudaStream_t s) {
  if (L.nfluid <= 0) return cudaSuccess;
  return launch_kernel(k_node_velocity_fluid<T>, dim3((L.nfluid + 255) / 256), dim3(256), 0, s, L.pdl, L);
}

template <typename T>
cudaError_t launch_node_velocity(const LbmView<T>& L, cudaStream_t s) {
  const dim3 g((unsigned)((L.N + 255) / 256));
  if (L.fast) return launch_kernel(k_node_velocity<T, true>, g, dim3(256), 0, s, L.pdl, L);
  return launch_kernel(k_node_velocity<T, false>, g, dim3(256), 0, s, L.pdl, L);
}

// Fluid readback: rho and u of every node (post-stream, force of the last collision).
template <typename T>
__global__ void k_moments(const LbmView<T> L, double* rho, double* u) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= L.N) return;
  const uint32_t m = L.nbmask[n];
  int X, Y, Z;
  node_xyz(n, L.nx, L.ny, X, Y, Z);
  T f[19];
  if (m & NB_SOLID) {
    for (int i = 0; i < 19; ++i) f[i] = L.fsrc[i * L.N + n];
  } else {
    pull(L, L.fsrc, X, Y, Z, n, m, f);
  }
  T rb = T(0);
  for (int i = 0; i < 19; ++i) rb += f[i];
  T rhoBar, jx, jy, jz, Fx, Fy, Fz;
  moments(f, rhoBar, jx, jy, jz);
  FieldLayout<T>::load(L.Fcur, L.N, n, Fx, Fy, Fz);
  const T r = T(1) + rhoBar;
  if (rho) rho[n] = 1.0 + (double)rb;
  if (u) {
    u[n] = (jx + T(0.5) * Fx) / r;
    u[L.N + n] = (jy + T(0.5) * Fy) / r;
    u[2 * L.N + n] = (jz + T(0.5) * Fz) / r;
  }
}
template <typename T>
cudaError_t launch_moments(const LbmView<T>& L, double* rho, double* u, cudaStream_t s) {
  k_moments<T><<<(unsigned)((L.N + 255) / 256), 256, 0, s>>>(L, rho, u);
  return cudaGetLastError();
}

// Post-stream populations (unshifted, double) of every node: the state a
// collide-then-stream solver holds between steps.  Wall nodes read w_i.
template <typename T>
__global__ void k_stream_out(const LbmView<T> L, double* out) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= L.N) return;
  const uint32_t m = L.nbmask[n];
  T f[19];
  if (m & NB_SOLID) {
    for (int i = 0; i < 19; ++i) f[i] = T(0);
  } else {
    int X, Y, Z;
    node_xyz(n, L.nx, L.ny, X, Y, Z);
    pull(L, L.fsrc, X, Y, Z, n, m, f);
  }
#pragma unroll
  for (int i = 0; i < 19; ++i) out[i * L.N + n] = (double)f[i] + wi(i);
}
template <typename T>
cudaError_t launch_stream_out(const LbmView<T>& L, double* out, cudaStream_t s) {
  k_stream_out<T><<<(unsigned)((L.N + 255) / 256), 256, 0, s>>>(L, out);
  return cudaGetLastError();
}

// Inverse of the pull: store post-collision values in L.fdst such that the
// next pull yields the given post-stream populations `in` (unshifted double
// [19][N]); with `in` null the populations are the equilibrium of (rho, u).
// Every stored slot has exactly one reader, so each is written once.
template <typename T>
__global__ void k_stream_in(const LbmView<T> L, const double* in, double rho, double ux, double uy, double uz) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= L.N) return;
  const uint32_t m = L.nbmask[n];
  const long long N = L.N;
  if (m & NB_SOLID) {
    for (int i = 0; i < 19; ++i) L.fdst[i * N + n] = T(0);
    return;
  }
  int X, Y, Z;
  node_xyz(n, L.nx, L.ny, X, Y, Z);
  const Nbr nb(X, Y, Z, L.nx, L.ny, L.nz);
  const uint32_t cls = m >> NB_CLASS_SHIFT;
  const double uu = ux * ux + uy * uy + uz * uz;
#pragma unroll
  for (int j = 0; j < 19; ++j) {
    double fj;
    if (in) {
      fj = in[j * N + n] - wi(j);
    } else {
      const double cu = cxi(j) * ux + cyi(j) * uy + czi(j) * uz;
      fj = wi(j) * ((rho - 1.0) + rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * uu));
    }
    if (j == 0) {
      L.fdst[n] = (T)fj;
      continue;
    }
    const int i = oppi(j);
    if (m & (1u << (i - 1))) {
      const uint32_t c = wall_class(L, i, X, Y, Z, nb, cls);
      const double cuw = cxi(i) * (double)L.uw[c][0] + cyi(i) * (double)L.uw[c][1] + czi(i) * (double)L.uw[c][2];
      L.fdst[i * N + n] = (T)(fj + 6.0 * wi(i) * cuw);
    } else {
      const int sx = cxi(j) > 0 ? nb.xm : (cxi(j) < 0 ? nb.xp : X);
      const int sy = cyi(j) > 0 ? nb.ym : (cyi(j) < 0 ? nb.yp : Y);
      const int sz = czi(j) > 0 ? nb.zm : (czi(j) < 0 ? nb.zp : Z);
      L.fdst[j * N + ((long long)sx + (long long)L.nx * ((long long)sy + (long long)L.ny * sz))] = (T)fj;
    }
  }
}
template <typename T>
cudaError_t launch_stream_in(const LbmView<T>& L, const double* in, double rho, const double* u3, cudaStream_t s) {
  k_stream_in<T><<<(unsigned)((L.N + 255) / 256), 256, 0, s>>>(L, in, rho, u3 ? u3[0] : 0.0, u3 ? u3[1] : 0.0,
                                                               u3 ? u3[2] : 0.0);
  return cudaGetLastError();
}

// force field <-> host layout [3][N] double
template <typename T>
__global__ void k_field_out(const T* F, double* out, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  T x, y, z;
  FieldLayout<T>::load(F, N, n, x, y, z);
  out[n] = x;
  out[N + n] = y;
  out[2 * N + n] = z;
}
template <typename T>
__global__ void k_field_in(const double* in, T* F, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  FieldLayout<T>::store(F, N, n, (T)in[n], (T)in[N + n], (T)in[2 * N + n]);
}
template <typename T>
__global__ void k_fill_body(T* F, const T* bodyz, long long plane, int nz, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int z = (int)(n / plane);
  FieldLayout<T>::store(F, N, n, bodyz[z], bodyz[nz + z], bodyz[2 * nz + z]);
}
// Copy of n 32-bit words from mapped pinned host memory into device memory
// by a kernel: a small per-step upload that does not wait behind a large
// device-to-host transfer on a copy engine.
__global__ void k_copy_words(uint32_t* dst, const uint32_t* src, int n) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = src[k];
}
cudaError_t launch_copy_words(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  const int n = (int)(bytes / 4);
  if (n <= 0) return cudaSuccess;
  k_copy_words<<<std::min((n + 255) / 256, 64), 256, 0, s>>>(static_cast<uint32_t*>(dst),
                                                             static_cast<const uint32_t*>(src), n);
  return cudaGetLastError();
}

// A changed body force applied to a force field that already holds the old
// one (and possibly the next step's spread): F += delta of its plane.
template <typename T>
__global__ void k_add_body(T* F, const T* dz, long long plane, int nz, long long N) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int z = (int)(n / plane);
  T x, y, w;
  FieldLayout<T>::load(F, N, n, x, y, w);
  FieldLayout<T>::store(F, N, n, x + dz[z], y + dz[nz + z], w + dz[2 * nz + z]);
}
template <typename T>
cudaError_t launch_add_body(T* F, const T* dz, long long plane, int nz, long long N, cudaStream_t s) {
  k_add_body<T><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(F, dz, plane, nz, N);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_field_out(const T* F, double* out, long long N, cudaStream_t s) {
  k_field_out<T><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(F, out, N);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_field_in(const double* in, T* F, long long N, cudaStream_t s) {
  k_field_in<T><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(in, F, N);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_fill_body(T* F, const T* bodyz, long long plane, int nz, long long N, cudaStream_t s) {
  k_fill_body<T><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(F, bodyz, plane, nz, N);
  return cudaGetLastError();
}
template <typename T>
size_t field_bytes(long long N) {
  return (size_t)N * FieldLayout<T>::kComps * sizeof(T);
}

// vector conversion T <-> double (vertex arrays)
template <typename T>
__global__ void k_convert_in(const double* src, T* dst, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = (T)src[k];
}
template <typename T>
cudaError_t launch_convert_in(const double* src, T* dst, long long n, cudaStream_t s) {
  k_convert_in<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, dst, n);
  return cudaGetLastError();
}

__global__ void k_bump_stamp(uint32_t* stamp) { *stamp += 1; }
cudaError_t launch_bump_stamp(uint32_t* stamp, cudaStream_t s) {
  k_bump_stamp<<<1, 1, 0, s>>>(stamp);
  return cudaGetLastError();
}

#define HC_LAT_INST(T)                                                                                    \
  template cudaError_t launch_collide_stream<T>(const LbmView<T>&, int, int, cudaStream_t);              \
  template bool make_bulk_plan<T>(int, int, int, int, int, BulkPlan*);                                    \
  template size_t bulk_smem_bytes<T>(const BulkPlan&);                                                     \
  template cudaError_t prepare_collide_bulk<T>(const BulkPlan&);                                           \
  template cudaError_t launch_collide_stream_bulk<T>(const LbmView<T>&, const BulkPlan&, cudaStream_t);   \
  template cudaError_t launch_node_velocity<T>(const LbmView<T>&, cudaStream_t);                         \
  template cudaError_t launch_node_velocity_fluid<T>(const LbmView<T>&, cudaStream_t);                   \
  template cudaError_t launch_node_velocity_packed<T>(const LbmView<T>&, cudaStream_t);                  \
  template cudaError_t launch_node_velocity_dense<T>(const LbmView<T>&, cudaStream_t);                   \
  template cudaError_t launch_collide_stream_fluid<T>(const LbmView<T>&, int, cudaStream_t);             \
  template cudaError_t launch_add_body<T>(T*, const T*, long long, int, long long, cudaStream_t);             \
  template cudaError_t launch_moments<T>(const LbmView<T>&, double*, double*, cudaStream_t);             \
  template cudaError_t launch_stream_out<T>(const LbmView<T>&, double*, cudaStream_t);                   \
  template cudaError_t launch_stream_in<T>(const LbmView<T>&, const double*, double, const double*,       \
                                           cudaStream_t);                                                \
  template cudaError_t launch_field_out<T>(const T*, double*, long long, cudaStream_t);                  \
  template cudaError_t launch_field_in<T>(const double*, T*, long long, cudaStream_t);                   \
  template cudaError_t launch_fill_body<T>(T*, const T*, long long, int, long long, cudaStream_t);       \
  template size_t field_bytes<T>(long long);                                                             \
  template cudaError_t launch_convert_in<T>(const double*, T*, long long, cudaStream_t);
HC_LAT_INST(double)
HC_LAT_INST(float)

}  // namespace hcd
