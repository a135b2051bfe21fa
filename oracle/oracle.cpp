// FP64 CPU oracle for the HemoCell IB-LBM time step.  TEST INFRASTRUCTURE:
// this is the checker the CUDA path is compared against; the product never
// links or calls it.  Every function cites the reference lines it restates.
// Parity with HemoCell itself is unpinned (its LBM core, Palabos, is not in
// the reference tree); see oracle.h.
//
// Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -shared -fPIC
// (-ffp-contract=off keeps x86-64 and aarch64 results identical).
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// D3Q19 lattice (Palabos ForcedD3Q19Descriptor, config/constant_defaults.h:58-61).
// Ordering: 0 rest, 1..9 "negative" half, i+9 the opposite of i.
const int C[19][3] = {{0, 0, 0},   {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0},
                      {-1, 1, 0},  {-1, 0, -1}, {-1, 0, 1}, {0, -1, -1}, {0, -1, 1},
                      {1, 0, 0},   {0, 1, 0},  {0, 0, 1},  {1, 1, 0},   {1, -1, 0},
                      {1, 0, 1},   {1, 0, -1}, {0, 1, 1},  {0, 1, -1}};
const double W[19] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                      1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 36,
                      1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
inline int opp(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }

// Saturation constants, config/constant_defaults.h:157-173.
const double MaxCellVolumetricChange = 0.01;
const double MaxCellSurfaceAreaChange = 0.09;
const double MaxCellBendingAngle = 0.0555;
const double MaxPLTBendingAngle = 2.467;
const double MaxCellPersistenceLength = 9.0;
const double FORCE_LIMIT = 50.0;  // constant_defaults.h:73-75 (pN, used raw in lattice units)

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3& operator+=(V3& a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3& operator-=(V3& a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
// helper/array.h:199-244
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double dot(V3 a, V3 b) {
  double r = 0;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
inline double norm(V3 a) {
  double r = 0;
  r += a.x * a.x;
  r += a.y * a.y;
  r += a.z * a.z;
  return std::sqrt(r);
}
// helper/array.h:271-285
inline void areaAndUnitNormal(V3 v0, V3 v1, V3 v2, double& area, V3& n) {
  V3 e01 = v1 - v0, e02 = v2 - v0;
  n = cross(e01, e02);
  double nn = norm(n);
  if (nn != 0.0) {
    area = 0.5 * nn;
    n = n / nn;
  } else {
    area = 0;
    n = {0, 0, 0};
  }
}
// helper/array.h:287-304 (isAreaWeighted == false)
inline V3 unitNormal(V3 v0, V3 v1, V3 v2) {
  V3 n = cross(v1 - v0, v2 - v0);
  double nn = norm(n);
  if (nn != 0) return n / nn;
  return {0, 0, 0};
}
// helper/geometryUtils.h:49-52
inline double angleBetweenFaces(V3 n1, V3 n2, V3 e) { return std::atan2(dot(cross(n1, n2), e), dot(n1, n2)); }

// ---------------------------------------------------------------------------
// CommonCellConstants (mechanics/commonCellConstants.cpp:70-409).
struct CellType {
  int model = 0;  // 0 RBC, 1 PLT, 2 WBC
  int nv = 0;
  std::vector<V3> rest;                 // template vertices (lattice units)
  std::vector<std::array<int, 3>> tris;
  std::vector<std::array<int, 2>> edges;
  std::vector<double> edge_l0, edge_angle0, tri_a0, patch_d0;
  std::vector<std::array<int, 2>> bend_tris, bend_outer;
  std::vector<std::array<int, 6>> ring;
  std::vector<int> ring_n;
  std::vector<std::array<int, 2>> inner;
  std::vector<double> inner_l0;
  double volume_eq = 0, area_mean_eq = 0, edge_mean_eq = 0, angle_mean_eq = 0;
  double k_link = 0, k_bend = 0, k_volume = 0, k_area = 0, eta_m = 0;
  double k_inner_rigid = 0, k_cyto = 0, core_radius = 0, radius = 0;
};

// Adjacent triangles of edge (a,b) with a<b: element [0] holds the triangle in
// which the edge runs b->a, element [1] the one in which it runs a->b.  This
// is the order under which the platelet dihedral force of
// mechanics/pltSimpleModel.cpp:156-182 is restoring on an outward-oriented mesh.
std::array<int, 2> adjacentTriangles(const CellType& t, int a, int b) {
  std::array<int, 2> r = {-1, -1};
  for (int k = 0; k < (int)t.tris.size(); ++k) {
    const auto& tr = t.tris[k];
    for (int c = 0; c < 3; ++c) {
      int p = tr[c], q = tr[(c + 1) % 3];
      if (p == b && q == a) r[0] = k;
      if (p == a && q == b) r[1] = k;
    }
  }
  return r;
}

// Third vertex of the triangle containing the directed edge a->b.
int nextAround(const CellType& t, int a, int b) {
  for (const auto& tr : t.tris)
    for (int c = 0; c < 3; ++c)
      if (tr[c] == a && tr[(c + 1) % 3] == b) return tr[(c + 2) % 3];
  return -1;
}

void buildConstants(CellType& t) {
  const std::vector<V3>& P = t.rest;
  // edges with i<j only (commonCellConstants.cpp:81-93)
  for (const auto& tr : t.tris) {
    if (tr[0] < tr[1]) t.edges.push_back({tr[0], tr[1]});
    if (tr[1] < tr[2]) t.edges.push_back({tr[1], tr[2]});
    if (tr[2] < tr[0]) t.edges.push_back({tr[2], tr[0]});
  }
  // rest lengths (:96-99)
  for (const auto& e : t.edges) t.edge_l0.push_back(norm(P[e[1]] - P[e[0]]));
  // rest dihedral angles (:102-140) and bending triangles/outer points (:174-189)
  for (const auto& e : t.edges) {
    std::array<int, 2> adj = adjacentTriangles(t, e[0], e[1]);
    const auto& A = t.tris[adj[0]];
    const auto& B = t.tris[adj[1]];
    V3 V1 = unitNormal(P[A[0]], P[A[1]], P[A[2]]);
    V3 V2 = unitNormal(P[B[0]], P[B[1]], P[B[2]]);
    V3 ev = P[e[1]] - P[e[0]];
    V3 uv = ev / norm(ev);
    t.edge_angle0.push_back(angleBetweenFaces(V1, V2, uv));
    t.bend_tris.push_back(adj);
    std::array<int, 2> op = {-1, -1};
    for (int i = 0; i < 3; ++i) {
      if (A[i] != e[0] && A[i] != e[1]) op[0] = A[i];
      if (B[i] != e[0] && B[i] != e[1]) op[1] = B[i];
    }
    t.bend_outer.push_back(op);
  }
  // inner edges (:143-161)
  for (const auto& e : t.inner) t.inner_l0.push_back(norm(P[e[1]] - P[e[0]]));
  // triangle rest areas (:164-167)
  for (const auto& tr : t.tris) {
    V3 n = cross(P[tr[1]] - P[tr[0]], P[tr[2]] - P[tr[0]]);
    t.tri_a0.push_back(0.5 * norm(n));
  }
  // volume_eq via MeshMetrics (helper/meshMetrics.h:148-184): every triangle
  // is visited once per corner vertex, in ascending triangle id per vertex.
  {
    std::vector<std::vector<int>> vtris(t.nv);
    for (int k = 0; k < (int)t.tris.size(); ++k)
      for (int c = 0; c < 3; ++c) vtris[t.tris[k][c]].push_back(k);
    double vol = 0;
    for (int v = 0; v < t.nv; ++v)
      for (int k : vtris[v]) {
        const auto& tr = t.tris[k];
        V3 tmp = cross(P[tr[1]], P[tr[2]]);
        double t6 = dot(P[tr[0]], tmp);
        vol += t6 / 6.0 / 3.0;
      }
    t.volume_eq = vol;
  }
  // means (:192-210)
  double s = 0;
  for (double a : t.tri_a0) s += a;
  t.area_mean_eq = s / t.tri_a0.size();
  s = 0;
  for (double l : t.edge_l0) s += l;
  t.edge_mean_eq = s / t.edge_l0.size();
  s = 0;
  for (double a : t.edge_angle0) s += a;
  t.angle_mean_eq = s / t.edge_angle0.size();
  // 1-ring, first from the edge list, then sorted around the vertex (:213-280)
  t.ring.assign(t.nv, {-1, -1, -1, -1, -1, -1});
  for (const auto& e : t.edges) {
    for (int k = 0; k < 6; ++k)
      if (t.ring[e[0]][k] == -1) { t.ring[e[0]][k] = e[1]; break; }
    for (int k = 0; k < 6; ++k)
      if (t.ring[e[1]][k] == -1) { t.ring[e[1]][k] = e[0]; break; }
  }
  t.ring_n.assign(t.nv, 0);
  for (int v = 0; v < t.nv; ++v)
    for (int k = 0; k < 6; ++k)
      if (t.ring[v][k] != -1) t.ring_n[v]++;
  for (int v = 0; v < t.nv; ++v) {
    int nvtx = t.ring[v][0];
    for (int n = 1; n < t.ring_n[v]; ++n) {
      nvtx = nextAround(t, v, nvtx);
      t.ring[v][n] = nvtx;
    }
  }
  // surface patch centre distance (:284-314)
  for (int i = 0; i < t.nv; ++i) {
    V3 sum = {0, 0, 0};
    for (int j = 0; j < t.ring_n[i]; ++j) sum += P[t.ring[i][j]];
    V3 mid = sum / (double)t.ring_n[i];
    V3 x = P[i];
    V3 dev = mid - x;
    V3 pn = {0, 0, 0};
    for (int j = 0; j < t.ring_n[i] - 1; ++j) {
      V3 tn = cross(P[t.ring[i][j]] - x, P[t.ring[i][j + 1]] - x);
      tn = tn / norm(tn);
      pn += tn;
    }
    V3 tn = cross(P[t.ring[i][t.ring_n[i] - 1]] - x, P[t.ring[i][0]] - x);
    tn = tn / norm(tn);
    pn += tn;
    pn = pn / norm(pn);
    t.patch_d0.push_back(dot(pn, dev));
  }
}

// ---------------------------------------------------------------------------
struct Cell {
  int type;
  int voff;  // first vertex in the global vertex arrays
  bool alive;
};

}  // namespace

struct orc_sim {
  int nx, ny, nz;
  int per[3];
  long N;
  double tau, omega, f_limit;
  std::vector<double> f, fnew;       // shifted populations f_i - w_i, SoA [19][N]
  std::vector<double> F, Fprev;      // force field [3][N]; Fprev = force of the last collision
  std::vector<uint8_t> flag;
  double uwall[256][3];
  int body_mode = 0;
  double body[3] = {0, 0, 0};
  std::vector<CellType> types;
  std::vector<Cell> cells;
  std::vector<V3> x, v, fv;          // vertex position, velocity, force
  std::vector<int> vcell;            // vertex -> cell
  std::vector<int> material_every;
  int velocity_every = 1;
  int iter = 0;
  std::vector<std::pair<int, V3>> ext;  // external vertex forces
  // IBM kernel cache of the last spread (core/hemoCellParticle.h:75-76)
  std::vector<std::vector<std::pair<long, double>>> kern;
  // repulsion (HemoCell::setRepulsion / enableBoundaryParticles,
  // core/hemoCell.cpp:420-436): constant, cutoff (lattice units), timescale
  double rep_const = 0, rep_cutoff = 0, brep_const = 0, brep_cutoff = 0;
  int rep_every = 0, brep_every = 0;  // 0 = disabled
  std::vector<V3> frep_cell, frep_wall;  // force_repulsion of each vertex, per source
  std::vector<long> boundary_nodes;       // populateBoundaryParticles

  long idx(long X, long Y, long Z) const { return X + nx * (Y + (long)ny * Z); }
  void bodyAt(long Z, double* b) const {
    if (body_mode == 1) {
      b[0] = body[0]; b[1] = body[1]; b[2] = body[2];
    } else if (body_mode == 2) {
      b[0] = body[0] * std::sin(2.0 * M_PI * (double)Z / (double)nz);
      b[1] = 0; b[2] = 0;
    } else {
      b[0] = b[1] = b[2] = 0;
    }
  }
};

namespace {

// Guo-forced BGK collide followed by streaming with (moving) bounce-back and
// periodic wrap: Palabos collideAndStream with GuoExternalForceBGKdynamics
// (core/hemoCell.cpp:317; dynamics chosen at examples/oneCellShear/oneCellShear.cpp:62-67).
// Populations are stored shifted by the lattice weights as Palabos does
// (rhoBar = rho - 1, core/hemoCellParticleField.cpp:955-957).
void collideStream(orc_sim* s) {
  const long N = s->N;
  const double om = s->omega;
  std::fill(s->fnew.begin(), s->fnew.end(), 0.0);
#pragma omp parallel for schedule(static)
  for (long Z = 0; Z < s->nz; ++Z) {
    for (long Y = 0; Y < s->ny; ++Y) {
      for (long X = 0; X < s->nx; ++X) {
        const long n = s->idx(X, Y, Z);
        if (s->flag[n] != 0) continue;
        double fb[19];
        for (int i = 0; i < 19; ++i) fb[i] = s->f[i * N + n];
        double rhoBar = 0;
        for (int i = 0; i < 19; ++i) rhoBar += fb[i];
        double j[3] = {0, 0, 0};
        for (int i = 0; i < 19; ++i) {
          j[0] += C[i][0] * fb[i];
          j[1] += C[i][1] * fb[i];
          j[2] += C[i][2] * fb[i];
        }
        const double rho = 1.0 + rhoBar;
        const double Fx = s->F[0 * N + n], Fy = s->F[1 * N + n], Fz = s->F[2 * N + n];
        // Guo: rho u = sum c f + F/2
        const double u[3] = {(j[0] + 0.5 * Fx) / rho, (j[1] + 0.5 * Fy) / rho, (j[2] + 0.5 * Fz) / rho};
        const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        for (int i = 0; i < 19; ++i) {
          const double cu = C[i][0] * u[0] + C[i][1] * u[1] + C[i][2] * u[2];
          const double feqBar = W[i] * (rhoBar + rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * uu));
          const double cmu[3] = {C[i][0] - u[0], C[i][1] - u[1], C[i][2] - u[2]};
          const double cF = C[i][0] * Fx + C[i][1] * Fy + C[i][2] * Fz;
          const double src = (1.0 - 0.5 * om) * W[i] *
                             (3.0 * (cmu[0] * Fx + cmu[1] * Fy + cmu[2] * Fz) + 9.0 * cu * cF);
          const double post = fb[i] - om * (fb[i] - feqBar) + src;
          // streaming
          long d[3] = {X + C[i][0], Y + C[i][1], Z + C[i][2]};
          const long dims[3] = {s->nx, s->ny, s->nz};
          bool outside = false;
          for (int a = 0; a < 3; ++a) {
            if (d[a] < 0 || d[a] >= dims[a]) {
              if (s->per[a]) d[a] = (d[a] + dims[a]) % dims[a];
              else outside = true;
            }
          }
          int cls = 0;
          bool bounce = outside;
          if (!outside) {
            cls = s->flag[s->idx(d[0], d[1], d[2])];
            bounce = cls != 0;
          }
          if (bounce) {
            // Ladd moving-wall bounce-back: f_opp = f*_i - 2 w_i rho0 (c_i . u_w)/cs^2, rho0 = 1
            const double* uw = s->uwall[cls];
            const double cuw = C[i][0] * uw[0] + C[i][1] * uw[1] + C[i][2] * uw[2];
            s->fnew[opp(i) * N + n] = post - 6.0 * W[i] * cuw;
          } else {
            s->fnew[i * N + s->idx(d[0], d[1], d[2])] = post;
          }
        }
      }
    }
  }
  s->f.swap(s->fnew);
}

// Velocity of a node as Palabos computeVelocity for the Guo dynamics
// (core/hemoCellParticleField.cpp:833): u = (sum c f + F/2) / rho.
void nodeVelocity(const orc_sim* s, long n, const std::vector<double>& F, double* u) {
  const long N = s->N;
  double rhoBar = 0, j[3] = {0, 0, 0};
  for (int i = 0; i < 19; ++i) rhoBar += s->f[i * N + n];
  for (int i = 0; i < 19; ++i) {
    const double fb = s->f[i * N + n];
    j[0] += C[i][0] * fb;
    j[1] += C[i][1] * fb;
    j[2] += C[i][2] * fb;
  }
  const double rho = 1.0 + rhoBar;
  for (int a = 0; a < 3; ++a) u[a] = (j[a] + 0.5 * F[a * N + n]) / rho;
}

// phi2 kernel, core/immersedBoundaryMethod.h:37-41
inline double phi2(double r) {
  r = std::fabs(r);
  r = 1.0 - r;
  return std::max(r, 0.0);
}

// interpolationCoefficientsPhi2, core/immersedBoundaryMethod.h:62-138, on one
// global periodic lattice: centre = floor(p + 0.5); nodes outside a
// non-periodic axis, zero-weight nodes and boundary nodes are skipped; the
// weights are renormalised to sum one.
void kernelWeights(const orc_sim* s, V3 p, std::vector<std::pair<long, double>>& out) {
  out.clear();
  const double P[3] = {p.x, p.y, p.z};
  const long dims[3] = {s->nx, s->ny, s->nz};
  long c[3];
  for (int a = 0; a < 3; ++a) c[a] = (long)std::floor(P[a] + 0.5);
  double total = 0;
  for (int dx = -1; dx < 2; ++dx)
    for (int dy = -1; dy < 2; ++dy)
      for (int dz = -1; dz < 2; ++dz) {
        long q[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
        long w[3];
        bool skip = false;
        for (int a = 0; a < 3; ++a) {
          w[a] = q[a];
          if (q[a] < 0 || q[a] >= dims[a]) {
            if (s->per[a]) w[a] = ((q[a] % dims[a]) + dims[a]) % dims[a];
            else skip = true;
          }
        }
        if (skip) continue;
        const double weight = phi2(P[0] - (double)q[0]) * phi2(P[1] - (double)q[1]) * phi2(P[2] - (double)q[2]);
        if (weight == 0.0) continue;
        const long n = s->idx(w[0], w[1], w[2]);
        if (s->flag[n] != 0) continue;
        total += weight;
        out.push_back({n, weight});
      }
  if (out.empty()) return;
  const double coeff = 1.0 / total;
  for (auto& pr : out) pr.second *= coeff;
}

// spreadParticleForce, core/hemoCellParticleField.cpp:841-863 (FORCE_LIMIT
// clamp :847-852 writes the clamped force back into the vertex).
void spread(orc_sim* s) {
  const long N = s->N;
  const int V = (int)s->x.size();
  for (const auto& e : s->ext) s->fv[e.first] += e.second;
  s->kern.resize(V);
  for (int i = 0; i < V; ++i) {
    if (!s->cells[s->vcell[i]].alive) { s->kern[i].clear(); continue; }
    kernelWeights(s, s->x[i], s->kern[i]);
    const double mag = norm(s->fv[i]);
    if (mag > s->f_limit) s->fv[i] = s->fv[i] * (s->f_limit / mag);
    V3 f = s->fv[i];
    if (i < (int)s->frep_cell.size()) f += s->frep_cell[i];
    if (i < (int)s->frep_wall.size()) f += s->frep_wall[i];
    for (const auto& pr : s->kern[i]) {
      s->F[0 * N + pr.first] += f.x * pr.second;
      s->F[1 * N + pr.first] += f.y * pr.second;
      s->F[2 * N + pr.first] += f.z * pr.second;
    }
  }
}

// Node of a position, int(x + 0.5) per axis (core/hemoCellParticleField.cpp:153-156),
// wrapped on periodic axes; false when it lies outside a bounded axis.
bool binNode(const orc_sim* s, const V3& p, long q[3]) {
  const double c[3] = {p.x, p.y, p.z};
  const long n[3] = {s->nx, s->ny, s->nz};
  for (int a = 0; a < 3; ++a) {
    long v = (long)std::floor(c[a] + 0.5);
    if (s->per[a]) v = ((v % n[a]) + n[a]) % n[a];
    else if (v < 0 || v >= n[a]) return false;
    q[a] = v;
  }
  return true;
}

// Separation a - b under the minimum-image convention on periodic axes.
V3 separation(const orc_sim* s, V3 d) {
  double c[3] = {d.x, d.y, d.z};
  const double n[3] = {(double)s->nx, (double)s->ny, (double)s->nz};
  for (int a = 0; a < 3; ++a)
    if (s->per[a]) c[a] -= n[a] * std::floor(c[a] / n[a] + 0.5);
  return {c[0], c[1], c[2]};
}

// applyRepulsionForce, core/hemoCellParticleField.cpp:677-743: vertices are
// binned per node; each node is paired with itself and its 13 forward
// neighbours, and every pair of vertices of different cells closer than the
// cutoff repels with r_const * (cutoff / d) along the separation (+ on the
// first, - on the second).  A node paired with itself visits each pair in both
// orders, so pairs sharing a node count twice, as in the reference.
void repulsionCells(orc_sim* s) {
  const int V = (int)s->x.size();
  s->frep_cell.assign(V, {0, 0, 0});
  std::map<long, std::vector<int>> grid;
  for (int i = 0; i < V; ++i) {
    if (!s->cells[s->vcell[i]].alive) continue;
    long q[3];
    if (binNode(s, s->x[i], q)) grid[s->idx(q[0], q[1], q[2])].push_back(i);
  }
  static const int D[14][3] = {{0, 0, 0},  {0, 1, 0},  {0, 0, 1},   {0, 1, 1},  {1, 0, 0},
                               {1, 1, 0},  {1, 0, 1},  {1, 1, 1},   {1, 0, -1}, {1, -1, 0},
                               {1, -1, -1}, {1, 1, -1}, {1, -1, 1}, {0, 1, -1}};
  const double rc = s->rep_cutoff, rk = s->rep_const;
  for (const auto& cell : grid) {
    const long n = cell.first;
    const long X = n % s->nx, Y = (n / s->nx) % s->ny, Z = n / ((long)s->nx * s->ny);
    for (const auto& d : D) {
      long q[3] = {X + d[0], Y + d[1], Z + d[2]};
      const long dims[3] = {s->nx, s->ny, s->nz};
      bool out = false;
      for (int a = 0; a < 3; ++a) {
        if (q[a] < 0 || q[a] >= dims[a]) {
          if (s->per[a]) q[a] = (q[a] + dims[a]) % dims[a];
          else out = true;
        }
      }
      if (out) continue;
      const auto it = grid.find(s->idx(q[0], q[1], q[2]));
      if (it == grid.end()) continue;
      for (int pi : cell.second)
        for (int qi : it->second) {
          if (pi == qi || s->vcell[pi] == s->vcell[qi]) continue;
          const V3 dv = separation(s, s->x[pi] - s->x[qi]);
          const double dist = norm(dv);
          if (dist < rc) {
            const V3 rfm = dv * (rk * (rc / dist) / dist);
            s->frep_cell[pi] += rfm;
            s->frep_cell[qi] = s->frep_cell[qi] - rfm;
          }
        }
    }
  }
}

// populateBoundaryParticles, core/hemoCellParticleField.cpp:865-889: wall
// nodes with a fluid node among their 26 neighbours.
void findBoundaryNodes(orc_sim* s) {
  s->boundary_nodes.clear();
  const long dims[3] = {s->nx, s->ny, s->nz};
  for (long Z = 0; Z < s->nz; ++Z)
    for (long Y = 0; Y < s->ny; ++Y)
      for (long X = 0; X < s->nx; ++X) {
        if (s->flag[s->idx(X, Y, Z)] == 0) continue;
        bool near_fluid = false;
        for (int dz = -1; dz <= 1 && !near_fluid; ++dz)
          for (int dy = -1; dy <= 1 && !near_fluid; ++dy)
            for (int dx = -1; dx <= 1 && !near_fluid; ++dx) {
              long q[3] = {X + dx, Y + dy, Z + dz};
              bool out = false;
              for (int a = 0; a < 3; ++a)
                if (q[a] < 0 || q[a] >= dims[a]) {
                  if (s->per[a]) q[a] = (q[a] + dims[a]) % dims[a];
                  else out = true;
                }
              if (!out && s->flag[s->idx(q[0], q[1], q[2])] == 0) near_fluid = true;
            }
        if (near_fluid) s->boundary_nodes.push_back(s->idx(X, Y, Z));
      }
}

// applyBoundaryRepulsionForce, core/hemoCellParticleField.cpp:891-918: a
// vertex binned within one node of a boundary node b and closer than the
// cutoff is pushed away from b with br_const * (cutoff / d).
void repulsionWalls(orc_sim* s) {
  const int V = (int)s->x.size();
  s->frep_wall.assign(V, {0, 0, 0});
  std::vector<char> is_b(s->N, 0);
  for (long b : s->boundary_nodes) is_b[b] = 1;
  const double rc = s->brep_cutoff, rk = s->brep_const;
  const long dims[3] = {s->nx, s->ny, s->nz};
  for (int i = 0; i < V; ++i) {
    if (!s->cells[s->vcell[i]].alive) continue;
    long q0[3];
    if (!binNode(s, s->x[i], q0)) continue;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          long q[3] = {q0[0] + dx, q0[1] + dy, q0[2] + dz};
          bool out = false;
          for (int a = 0; a < 3; ++a)
            if (q[a] < 0 || q[a] >= dims[a]) {
              if (s->per[a]) q[a] = (q[a] + dims[a]) % dims[a];
              else out = true;
            }
          if (out || !is_b[s->idx(q[0], q[1], q[2])]) continue;
          const V3 dv = separation(s, s->x[i] - V3{(double)q[0], (double)q[1], (double)q[2]});
          const double dist = norm(dv);
          if (dist < rc) s->frep_wall[i] += dv * (rk * (rc / dist) / dist);
        }
  }
}

// The repulsion terms due at this step (core/hemoCell.cpp:307-312).  Each
// term is recomputed at its own timescale and kept in between.
void repulsion(orc_sim* s) {
  if (s->rep_every > 0 && s->iter % s->rep_every == 0) repulsionCells(s);
  if (s->brep_every > 0 && s->iter % s->brep_every == 0) repulsionWalls(s);
}

// interpolateFluidVelocity, core/hemoCellParticleField.cpp:819-839, with the
// kernel cached by the spread of the same step (:827).  The velocity uses the
// force of this step's collision (Fprev): the reference resets the force
// field only at the end of iterate() (core/hemoCell.cpp:369), and nothing
// between the collision and that reset writes it, so resetting right after
// the collision and keeping the old field is the same computation.
void interpolate(orc_sim* s) {
  const int V = (int)s->x.size();
  if ((int)s->kern.size() != V) {
    s->kern.resize(V);
    for (int i = 0; i < V; ++i) kernelWeights(s, s->x[i], s->kern[i]);
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < V; ++i) {
    if (!s->cells[s->vcell[i]].alive) continue;
    V3 vel = {0, 0, 0};
    for (const auto& pr : s->kern[i]) {
      double u[3];
      nodeVelocity(s, pr.first, s->Fprev, u);
      vel += V3{u[0], u[1], u[2]} * pr.second;
    }
    s->v[i] = vel;
  }
}

// advanceParticles: Euler x += v (core/hemoCellParticle.h:188-203) and wall
// check on the nearest node (core/hemoCellParticleField.cpp:566-588).  A cell
// with a vertex on a boundary node is removed whole.
void advance(orc_sim* s) {
  const int V = (int)s->x.size();
  const long dims[3] = {s->nx, s->ny, s->nz};
  std::vector<int> hit;
  for (int i = 0; i < V; ++i) {
    const Cell& c = s->cells[s->vcell[i]];
    if (!c.alive) continue;
    s->x[i] += s->v[i];
    const double P[3] = {s->x[i].x, s->x[i].y, s->x[i].z};
    long q[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
      q[a] = (long)std::floor(P[a] + 0.5);
      if (q[a] < 0 || q[a] >= dims[a]) {
        if (s->per[a]) q[a] = ((q[a] % dims[a]) + dims[a]) % dims[a];
        else inside = false;
      }
    }
    if (inside && s->flag[s->idx(q[0], q[1], q[2])] != 0) hit.push_back(s->vcell[i]);
  }
  for (int c : hit) s->cells[c].alive = false;
}

// --- constitutive models --------------------------------------------------
// rbcHighOrderModel.cpp:38-207 (model 0) and wbcHighOrderModel.cpp:42-225 (model 2)
// The volume is the reference's six-term triple-product sum
// (rbcHighOrderModel.cpp:62-68) evaluated on coordinates relative to the
// cell's vertex 0: a closed surface's signed volume does not depend on the
// origin, and on absolute coordinates the sum cancels by orders of magnitude
// (a platelet 30 lu from the origin loses ~13 digits).
inline double faceVolume6(V3 o, V3 p0, V3 p1, V3 p2) {
  const V3 v0 = p0 - o, v1 = p1 - o, v2 = p2 - o;
  const double v210 = v2.x * v1.y * v0.z;
  const double v120 = v1.x * v2.y * v0.z;
  const double v201 = v2.x * v0.y * v1.z;
  const double v021 = v0.x * v2.y * v1.z;
  const double v102 = v1.x * v0.y * v2.z;
  const double v012 = v0.x * v1.y * v2.z;
  return (-v210 + v120 + v201 - v021 - v102 + v012);
}

void mechanicsHighOrder(orc_sim* s, const CellType& t, const Cell& c) {
  V3* X = &s->x[c.voff];
  V3* Vv = &s->v[c.voff];
  V3* Fo = &s->fv[c.voff];
  double volume = 0.0;
  std::vector<double> areas;
  std::vector<V3> normals;
  areas.reserve(t.tris.size());
  normals.reserve(t.tris.size());
  int tn = 0;
  for (const auto& tr : t.tris) {
    const V3 v0 = X[tr[0]], v1 = X[tr[1]], v2 = X[tr[2]];
    volume += faceVolume6(X[0], v0, v1, v2);
    double area;
    V3 nrm;
    areaAndUnitNormal(v0, v1, v2, area, nrm);
    const double ar = (area - t.tri_a0[tn]) / t.tri_a0[tn];
    const double afm = t.k_area * (ar + ar / std::fabs(MaxCellSurfaceAreaChange - ar * ar));
    V3 cen = {(v0.x + v1.x + v2.x) / 3.0, (v0.y + v1.y + v2.y) / 3.0, (v0.z + v1.z + v2.z) / 3.0};
    Fo[tr[0]] += afm * (cen - v0);
    Fo[tr[1]] += afm * (cen - v1);
    Fo[tr[2]] += afm * (cen - v2);
    areas.push_back(area);
    normals.push_back(nrm);
    tn++;
  }
  volume *= (1.0 / 6.0);
  const double vf = (volume - t.volume_eq) / t.volume_eq;
  const double vforce = -t.k_volume * vf / std::fabs(MaxCellVolumetricChange - vf * vf);
  tn = 0;
  for (const auto& tr : t.tris) {
    const V3 lvf = (vforce * normals[tn]) * (areas[tn] / t.area_mean_eq);
    Fo[tr[0]] += lvf;
    Fo[tr[1]] += lvf;
    Fo[tr[2]] += lvf;
    tn++;
  }
  // per-vertex bending (rbcHighOrderModel.cpp:127-166)
  for (int i = 0; i < t.nv; ++i) {
    const int rn = t.ring_n[i];
    V3 sum = {0, 0, 0};
    for (int j = 0; j < rn; ++j) sum += X[t.ring[i][j]];
    const V3 mid = sum / (double)rn;
    const V3 dev = mid - X[i];
    V3 pn = {0, 0, 0};
    for (int j = 0; j < rn - 1; ++j) {
      V3 tnrm = cross(X[t.ring[i][j]] - X[i], X[t.ring[i][j + 1]] - X[i]);
      tnrm = tnrm / norm(tnrm);
      pn += tnrm;
    }
    V3 tnrm = cross(X[t.ring[i][rn - 1]] - X[i], X[t.ring[i][0]] - X[i]);
    tnrm = tnrm / norm(tnrm);
    pn += tnrm;
    pn = pn / norm(pn);
    const double ndev = dot(pn, dev);
    const double dDev = (ndev - t.patch_d0[i]) / t.edge_mean_eq;
    const V3 bf = t.k_bend * (dDev + dDev / std::fabs(MaxCellBendingAngle - dDev * dDev)) * pn;
    Fo[i] += bf;
    const V3 nbf = (-1.0 * bf) / (double)rn;
    for (int j = 0; j < rn; ++j) Fo[t.ring[i][j]] += nbf;
  }
  // per-edge link + membrane viscosity (rbcHighOrderModel.cpp:170-204; the
  // WBC applies viscosity unconditionally, wbcHighOrderModel.cpp:183-196)
  int en = 0;
  for (const auto& e : t.edges) {
    const V3 p0 = X[e[0]], p1 = X[e[1]];
    const V3 ev = p1 - p0;
    const double L = norm(ev);
    const V3 uv = ev / L;
    const double ef = (L - t.edge_l0[en]) / t.edge_l0[en];
    const double fs = t.k_link * (ef + ef / std::fabs(MaxCellPersistenceLength - ef * ef));
    const V3 force = uv * fs;
    Fo[e[0]] += force;
    Fo[e[1]] -= force;
    if (t.model == 2 || t.eta_m != 0.0) {
      const V3 rv = Vv[e[1]] - Vv[e[0]];
      V3 fvisc = t.eta_m * (dot(rv, uv) * uv);
      const double m = norm(fvisc);
      if (m > FORCE_LIMIT / 4.0) fvisc = fvisc * ((FORCE_LIMIT / 4.0) / m);
      Fo[e[0]] += fvisc;
      Fo[e[1]] -= fvisc;
    }
    en++;
  }
  if (t.model == 2) {
    // rigid inner core and cytoskeleton links (wbcHighOrderModel.cpp:202-223)
    for (const auto& e : t.inner) {
      const V3 p0 = X[e[0]], p1 = X[e[1]];
      const V3 ev = p1 - p0;
      const double L = norm(ev);
      const V3 uv = ev / L;
      if (L < 2 * t.radius) {
        const V3 force = uv * (1.0 - (L / (2 * t.radius))) * t.k_cyto;
        Fo[e[0]] -= force;
        Fo[e[1]] += force;
      }
      if (L < 2 * t.core_radius) {
        const V3 force = uv * (1 - (L / (2 * t.core_radius))) * t.k_inner_rigid;
        Fo[e[0]] -= force;
        Fo[e[1]] += force;
      }
    }
  }
}

// pltSimpleModel.cpp:44-208
void mechanicsPlt(orc_sim* s, const CellType& t, const Cell& c) {
  V3* X = &s->x[c.voff];
  V3* Vv = &s->v[c.voff];
  V3* Fo = &s->fv[c.voff];
  double volume = 0.0;
  std::vector<double> areas;
  std::vector<V3> normals;
  int tn = 0;
  for (const auto& tr : t.tris) {
    const V3 v0 = X[tr[0]], v1 = X[tr[1]], v2 = X[tr[2]];
    volume += faceVolume6(X[0], v0, v1, v2);
    double area;
    V3 nrm;
    areaAndUnitNormal(v0, v1, v2, area, nrm);
    const double ar = (area - t.tri_a0[tn]) / t.tri_a0[tn];
    const double afm = t.k_area * (ar + ar / std::fabs(MaxCellSurfaceAreaChange - ar * ar));
    V3 cen = {(v0.x + v1.x + v2.x) / 3.0, (v0.y + v1.y + v2.y) / 3.0, (v0.z + v1.z + v2.z) / 3.0};
    Fo[tr[0]] += afm * (cen - v0);
    Fo[tr[1]] += afm * (cen - v1);
    Fo[tr[2]] += afm * (cen - v2);
    areas.push_back(area);
    normals.push_back(nrm);
    tn++;
  }
  volume *= (1.0 / 6.0);
  const double vf = (volume - t.volume_eq) / t.volume_eq;
  const double vforce = -t.k_volume * vf / std::fabs(MaxCellVolumetricChange - vf * vf);
  tn = 0;
  for (const auto& tr : t.tris) {
    const V3 lvf = (vforce * normals[tn]) * (areas[tn] / t.area_mean_eq);
    Fo[tr[0]] += lvf;
    Fo[tr[1]] += lvf;
    Fo[tr[2]] += lvf;
    tn++;
  }
  int en = 0;
  for (const auto& e : t.edges) {
    const V3 v0 = X[e[0]], v1 = X[e[1]];
    const V3 ev = v1 - v0;
    const double L = std::sqrt(ev.x * ev.x + ev.y * ev.y + ev.z * ev.z);
    const V3 uv = ev / L;
    const double ef = (L - t.edge_l0[en]) / t.edge_l0[en];
    const double fs = t.k_link * (ef + ef / std::fabs(MaxCellPersistenceLength - ef * ef));
    const V3 force = uv * fs;
    Fo[e[0]] += force;
    Fo[e[1]] -= force;
    // always-on membrane viscosity (:140-153)
    const V3 rv = Vv[e[1]] - Vv[e[0]];
    V3 fvisc = t.eta_m * (dot(rv, uv) * uv);
    const double m = norm(fvisc);
    if (m > FORCE_LIMIT / 4.0) fvisc = fvisc * ((FORCE_LIMIT / 4.0) / m);
    Fo[e[0]] += fvisc;
    Fo[e[1]] -= fvisc;
    // dihedral bending (:156-182)
    const auto& A = t.tris[t.bend_tris[en][0]];
    const auto& B = t.tris[t.bend_tris[en][1]];
    const V3 V1 = unitNormal(X[A[0]], X[A[1]], X[A[2]]);
    const V3 V2 = unitNormal(X[B[0]], X[B[1]], X[B[2]]);
    const double angle = angleBetweenFaces(V1, V2, uv);
    const double af = angle - t.edge_angle0[en];
    const double fm = t.k_bend * (af + af / std::fabs(MaxPLTBendingAngle - af * af));
    const V3 bf = fm * (V1 + V2) * 0.5;
    Fo[e[0]] += bf;
    Fo[e[1]] += bf;
    Fo[t.bend_outer[en][0]] -= bf;
    Fo[t.bend_outer[en][1]] -= bf;
    en++;
  }
  // inner links (:188-205)
  int in = 0;
  for (const auto& e : t.inner) {
    const V3 v0 = X[e[0]], v1 = X[e[1]];
    const V3 ev = v1 - v0;
    const double L = std::sqrt(ev.x * ev.x + ev.y * ev.y + ev.z * ev.z);
    const V3 uv = ev / L;
    const double ef = (L - t.inner_l0[in]) / t.inner_l0[in];
    const double fs = t.k_link * 5.0 * ef;
    const V3 force = uv * fs;
    Fo[e[0]] += force;
    Fo[e[1]] -= force;
    in++;
  }
}

// applyConstitutiveModel, core/hemoCellParticleField.cpp:633-675: per type
// due this step, zero the forces of its vertices, then run the model on every
// complete cell.
void mechanics(orc_sim* s, bool forced) {
  const int nt = (int)s->types.size();
  for (int ty = 0; ty < nt; ++ty) {
    const int every = s->material_every.empty() ? 1 : s->material_every[ty];
    if (!(forced || s->iter % every == 0)) continue;
    const CellType& t = s->types[ty];
#pragma omp parallel for schedule(dynamic)
    for (int ci = 0; ci < (int)s->cells.size(); ++ci) {
      const Cell& c = s->cells[ci];
      if (c.type != ty) continue;
      for (int k = 0; k < t.nv; ++k) s->fv[c.voff + k] = {0, 0, 0};
      if (!c.alive) continue;
      if (t.model == 1) mechanicsPlt(s, t, c);
      else mechanicsHighOrder(s, t, c);
    }
  }
}

// setExternalVector reset (core/hemoCell.cpp:367-372) followed by the
// driver's body force (examples/pipeflow/pipeflow.cpp:141-146).  The force
// of the collision just done is kept for readback and interpolation.
void resetForce(orc_sim* s, bool keep = true) {
  const long N = s->N;
  if (keep) s->Fprev = s->F;
  for (long Z = 0; Z < s->nz; ++Z) {
    double b[3];
    s->bodyAt(Z, b);
    for (long Y = 0; Y < s->ny; ++Y)
      for (long X = 0; X < s->nx; ++X) {
        const long n = s->idx(X, Y, Z);
        for (int a = 0; a < 3; ++a) s->F[a * N + n] = b[a];
      }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

orc_sim* orc_create(int nx, int ny, int nz, int px, int py, int pz, double tau, double f_limit) {
  orc_sim* s = new orc_sim();
  s->nx = nx; s->ny = ny; s->nz = nz;
  s->per[0] = px; s->per[1] = py; s->per[2] = pz;
  s->N = (long)nx * ny * nz;
  s->tau = tau;
  s->omega = 1.0 / tau;
  s->f_limit = f_limit;
  s->f.assign(19 * s->N, 0.0);
  s->fnew.assign(19 * s->N, 0.0);
  s->F.assign(3 * s->N, 0.0);
  s->Fprev.assign(3 * s->N, 0.0);
  s->flag.assign(s->N, 0);
  std::memset(s->uwall, 0, sizeof(s->uwall));
  return s;
}
void orc_destroy(orc_sim* s) { delete s; }
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
void orc_set_flags(orc_sim* s, const uint8_t* flags) { std::memcpy(s->flag.data(), flags, s->N); }
void orc_set_wall_velocity(orc_sim* s, int cls, const double* u3) {
  for (int a = 0; a < 3; ++a) s->uwall[cls & 255][a] = u3[a];
}
void orc_set_body_force(orc_sim* s, int mode, const double* p) {
  s->body_mode = mode;
  for (int a = 0; a < 3; ++a) s->body[a] = p ? p[a] : 0.0;
  // the force field holds the body force from the start (driver sets it before iterate)
  resetForce(s, false);
}
// lattice.initialize() at rest / initializeAtEquilibrium (core/hemoCell.cpp:132)
void orc_init_equilibrium(orc_sim* s, double rho, const double* u3) {
  const long N = s->N;
  const double u[3] = {u3 ? u3[0] : 0.0, u3 ? u3[1] : 0.0, u3 ? u3[2] : 0.0};
  const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  for (long n = 0; n < N; ++n)
    for (int i = 0; i < 19; ++i) {
      if (s->flag[n] != 0) { s->f[i * N + n] = 0; continue; }
      const double cu = C[i][0] * u[0] + C[i][1] * u[1] + C[i][2] * u[2];
      s->f[i * N + n] = W[i] * ((rho - 1.0) + rho * (3.0 * cu + 4.5 * cu * cu - 1.5 * uu));
    }
}

int orc_add_cell_type(orc_sim* s, int model, int nv, const double* xyz, int nf, const int* tris, int ni,
                      const int* inner, const double* k) {
  CellType t;
  t.model = model;
  t.nv = nv;
  for (int i = 0; i < nv; ++i) t.rest.push_back({xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
  for (int i = 0; i < nf; ++i) t.tris.push_back({tris[3 * i], tris[3 * i + 1], tris[3 * i + 2]});
  for (int i = 0; i < ni; ++i) t.inner.push_back({inner[2 * i], inner[2 * i + 1]});
  t.k_link = k[0]; t.k_bend = k[1]; t.k_volume = k[2]; t.k_area = k[3]; t.eta_m = k[4];
  t.k_inner_rigid = k[5]; t.k_cyto = k[6]; t.core_radius = k[7]; t.radius = k[8];
  buildConstants(t);
  s->types.push_back(std::move(t));
  s->material_every.push_back(1);
  return (int)s->types.size() - 1;
}

int orc_add_cell(orc_sim* s, int type, const double* xyz) {
  const CellType& t = s->types[type];
  Cell c;
  c.type = type;
  c.voff = (int)s->x.size();
  c.alive = true;
  const int cid = (int)s->cells.size();
  for (int i = 0; i < t.nv; ++i) {
    s->x.push_back({xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
    s->v.push_back({0, 0, 0});
    s->fv.push_back({0, 0, 0});
    s->vcell.push_back(cid);
  }
  s->cells.push_back(c);
  s->kern.clear();
  return cid;
}

void orc_set_timescales(orc_sim* s, const int* material_every, int velocity_every) {
  for (size_t i = 0; i < s->material_every.size(); ++i) s->material_every[i] = material_every[i];
  s->velocity_every = velocity_every;
}

void orc_set_vertex_forces(orc_sim* s, int n, const int* ids, const double* forces) {
  s->ext.clear();
  for (int k = 0; k < n; ++k) s->ext.push_back({ids[k], V3{forces[3 * k], forces[3 * k + 1], forces[3 * k + 2]}});
}

// setRepulsion / enableBoundaryParticles (core/hemoCell.cpp:420-436); cutoffs
// in lattice units, every <= 0 disables the term
void orc_set_repulsion(orc_sim* s, double k, double cutoff, int every) {
  s->rep_const = k;
  s->rep_cutoff = cutoff;
  s->rep_every = every > 0 ? every : 0;
  if (s->rep_every == 0) s->frep_cell.clear();
}
void orc_set_boundary_repulsion(orc_sim* s, double k, double cutoff, int every) {
  s->brep_const = k;
  s->brep_cutoff = cutoff;
  s->brep_every = every > 0 ? every : 0;
  if (s->brep_every == 0) s->frep_wall.clear();
  else findBoundaryNodes(s);
}
void orc_stage_repulsion(orc_sim* s) {
  if (s->rep_every > 0) repulsionCells(s);
  if (s->brep_every > 0) repulsionWalls(s);
}
void orc_read_repulsion(orc_sim* s, double* f) {
  const int V = (int)s->x.size();
  for (int i = 0; i < V; ++i) {
    V3 r = {0, 0, 0};
    if (i < (int)s->frep_cell.size()) r += s->frep_cell[i];
    if (i < (int)s->frep_wall.size()) r += s->frep_wall[i];
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
  }
}

void orc_stage_spread(orc_sim* s) { spread(s); }
void orc_stage_collide_stream(orc_sim* s) {
  collideStream(s);
  resetForce(s);
}
void orc_stage_interpolate(orc_sim* s) { interpolate(s); }
void orc_stage_advance(orc_sim* s) { advance(s); }
void orc_stage_mechanics(orc_sim* s, int forced) { mechanics(s, forced != 0); }

// HemoCell::iterate, core/hemoCell.cpp:299-376 (CEPAC, solidify and
// interior viscosity are not part of this path).
void orc_step(orc_sim* s, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    repulsion(s);
    spread(s);
    collideStream(s);
    resetForce(s);
    if (s->iter % s->velocity_every == 0) interpolate(s);
    advance(s);
    mechanics(s, false);
    s->iter++;
  }
}

long orc_num_nodes(orc_sim* s) { return s->N; }
int orc_num_vertices(orc_sim* s) { return (int)s->x.size(); }
int orc_num_cells(orc_sim* s) { return (int)s->cells.size(); }
int orc_iter(orc_sim* s) { return s->iter; }

void orc_read_fluid(orc_sim* s, double* rho, double* u) {
  const long N = s->N;
  for (long n = 0; n < N; ++n) {
    double rb = 0;
    for (int i = 0; i < 19; ++i) rb += s->f[i * N + n];
    double uu[3];
    nodeVelocity(s, n, s->Fprev, uu);
    if (rho) rho[n] = 1.0 + rb;
    if (u) for (int a = 0; a < 3; ++a) u[a * N + n] = uu[a];
  }
}
void orc_read_populations(orc_sim* s, double* f) {
  const long N = s->N;
  for (int i = 0; i < 19; ++i)
    for (long n = 0; n < N; ++n) f[i * N + n] = s->f[i * N + n] + W[i];
}
void orc_write_populations(orc_sim* s, const double* f) {
  const long N = s->N;
  for (int i = 0; i < 19; ++i)
    for (long n = 0; n < N; ++n) s->f[i * N + n] = f[i * N + n] - W[i];
}
void orc_read_force_field(orc_sim* s, double* F, int which) {
  const std::vector<double>& src = which ? s->Fprev : s->F;
  std::memcpy(F, src.data(), sizeof(double) * 3 * s->N);
}
void orc_write_force_field(orc_sim* s, const double* F) {
  std::memcpy(s->F.data(), F, sizeof(double) * 3 * s->N);
  s->Fprev = s->F;
}
void orc_read_vertices(orc_sim* s, double* x, double* v, double* f) {
  for (size_t i = 0; i < s->x.size(); ++i) {
    if (x) { x[3 * i] = s->x[i].x; x[3 * i + 1] = s->x[i].y; x[3 * i + 2] = s->x[i].z; }
    if (v) { v[3 * i] = s->v[i].x; v[3 * i + 1] = s->v[i].y; v[3 * i + 2] = s->v[i].z; }
    if (f) { f[3 * i] = s->fv[i].x; f[3 * i + 1] = s->fv[i].y; f[3 * i + 2] = s->fv[i].z; }
  }
}
void orc_write_vertices(orc_sim* s, const double* x, const double* v, const double* f) {
  for (size_t i = 0; i < s->x.size(); ++i) {
    if (x) s->x[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    if (v) s->v[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    if (f) s->fv[i] = {f[3 * i], f[3 * i + 1], f[3 * i + 2]};
  }
  s->kern.clear();
}
void orc_read_cells(orc_sim* s, int* alive, double* volume) {
  for (size_t ci = 0; ci < s->cells.size(); ++ci) {
    const Cell& c = s->cells[ci];
    if (alive) alive[ci] = c.alive ? 1 : 0;
    if (volume) {
      const CellType& t = s->types[c.type];
      double vol = 0;
      for (const auto& tr : t.tris)
        vol += faceVolume6(s->x[c.voff], s->x[c.voff + tr[0]], s->x[c.voff + tr[1]], s->x[c.voff + tr[2]]);
      volume[ci] = vol / 6.0;
    }
  }
}

// Binning and neighbour lists (update_pg core/hemoCellParticleField.cpp:137-168,
// ownership isContainedABS core/hemoCellParticleField.h:93-103) restated for
// one global lattice: bin = floor(x+0.5) wrapped, tile = bin / tile dims,
// CSR sorted by (tile, cell, vertex).
int orc_bins(orc_sim* s, int tx, int ty, int tz, const double* xin, int* vertex_node, int* vertex_tile,
             int* tile_offsets, int* tile_vertices, int* tile_cell_offsets, int* tile_cells, int max_tile_cells) {
  const long dims[3] = {s->nx, s->ny, s->nz};
  const int td[3] = {tx, ty, tz};
  const int nt[3] = {(s->nx + tx - 1) / tx, (s->ny + ty - 1) / ty, (s->nz + tz - 1) / tz};
  const int ntiles = nt[0] * nt[1] * nt[2];
  const int V = (int)s->x.size();
  std::vector<std::vector<int>> lists(ntiles);
  for (int i = 0; i < V; ++i) {
    const double P[3] = {xin ? xin[3 * i] : s->x[i].x, xin ? xin[3 * i + 1] : s->x[i].y,
                         xin ? xin[3 * i + 2] : s->x[i].z};
    long q[3];
    bool inside = s->cells[s->vcell[i]].alive;
    for (int a = 0; a < 3; ++a) {
      q[a] = (long)std::floor(P[a] + 0.5);
      if (q[a] < 0 || q[a] >= dims[a]) {
        if (s->per[a]) q[a] = ((q[a] % dims[a]) + dims[a]) % dims[a];
        else inside = false;
      }
    }
    if (!inside) { vertex_node[i] = -1; vertex_tile[i] = -1; continue; }
    vertex_node[i] = (int)s->idx(q[0], q[1], q[2]);
    const int t = (int)(q[0] / td[0] + nt[0] * (q[1] / td[1] + nt[1] * (q[2] / td[2])));
    vertex_tile[i] = t;
    lists[t].push_back(i);  // vertex ids grow with (cell, vertex), so each list is sorted
  }
  int off = 0, coff = 0;
  for (int t = 0; t < ntiles; ++t) {
    tile_offsets[t] = off;
    tile_cell_offsets[t] = coff;
    int last = -1;
    for (int i : lists[t]) {
      tile_vertices[off++] = i;
      if (s->vcell[i] != last) {
        if (coff >= max_tile_cells) return -1;
        tile_cells[coff++] = s->vcell[i];
        last = s->vcell[i];
      }
    }
  }
  tile_offsets[ntiles] = off;
  tile_cell_offsets[ntiles] = coff;
  return ntiles;
}

// Neighbour lists: for each tile, the cells with vertices in it or in one of
// its 26 neighbouring tiles (block neighbours core/hemoCellFields.cpp:230-236,
// here tiles of one global lattice), wrapped on periodic axes, as sorted
// distinct ids in CSR.  Input: the tile cell lists of orc_bins.
int orc_neighbours(int ntx, int nty, int ntz, int px, int py, int pz, const int* tile_cell_offsets,
                   const int* tile_cells, int* nb_offsets, int* nb_cells, int max_cells) {
  const int n3[3] = {ntx, nty, ntz}, per[3] = {px, py, pz};
  const int ntiles = ntx * nty * ntz;
  int off = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int c0[3] = {t % ntx, (t / ntx) % nty, t / (ntx * nty)};
    std::set<int> tiles, cells;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          int c[3] = {c0[0] + dx, c0[1] + dy, c0[2] + dz};
          bool ok = true;
          for (int a = 0; a < 3; ++a)
            if (c[a] < 0 || c[a] >= n3[a]) {
              if (per[a]) c[a] = (c[a] + n3[a]) % n3[a];
              else ok = false;
            }
          if (ok) tiles.insert(c[0] + ntx * (c[1] + nty * c[2]));
        }
    for (int u : tiles)
      for (int k = tile_cell_offsets[u]; k < tile_cell_offsets[u + 1]; ++k) cells.insert(tile_cells[k]);
    nb_offsets[t] = off;
    for (int c : cells) {
      if (off >= max_cells) return -1;
      nb_cells[off++] = c;
    }
  }
  nb_offsets[ntiles] = off;
  return ntiles;
}

int orc_type_sizes(orc_sim* s, int type, int* out4) {
  const CellType& t = s->types[type];
  out4[0] = t.nv;
  out4[1] = (int)t.tris.size();
  out4[2] = (int)t.edges.size();
  out4[3] = (int)t.inner.size();
  return 0;
}
void orc_type_constants(orc_sim* s, int type, int* edges, double* edge_l0, double* edge_angle0, int* ring,
                        int* ring_n, double* patch_d0, double* tri_a0, int* bend_outer, double* scalars) {
  const CellType& t = s->types[type];
  for (size_t e = 0; e < t.edges.size(); ++e) {
    edges[2 * e] = t.edges[e][0];
    edges[2 * e + 1] = t.edges[e][1];
    edge_l0[e] = t.edge_l0[e];
    edge_angle0[e] = t.edge_angle0[e];
    bend_outer[2 * e] = t.bend_outer[e][0];
    bend_outer[2 * e + 1] = t.bend_outer[e][1];
  }
  for (int v = 0; v < t.nv; ++v) {
    for (int k = 0; k < 6; ++k) ring[6 * v + k] = t.ring[v][k];
    ring_n[v] = t.ring_n[v];
    patch_d0[v] = t.patch_d0[v];
  }
  for (size_t k = 0; k < t.tris.size(); ++k) tri_a0[k] = t.tri_a0[k];
  scalars[0] = t.volume_eq;
  scalars[1] = t.area_mean_eq;
  scalars[2] = t.edge_mean_eq;
  scalars[3] = t.angle_mean_eq;
}

// Parameters::lbm_base_parameters, mechanics/constantConversion.cpp:36-59.
// tau_override > 0 fixes tau (and nu_lbm) the way the dt<0 branch does.
void orc_units(double dx, double dt, double nu_p, double rho_p, double kBT_p, double tau_override, double* out) {
  double tau, nu_lbm;
  if (tau_override > 0) {
    tau = tau_override;
    nu_lbm = 1.0 / 3.0 * (tau - 0.5);
  } else {
    nu_lbm = nu_p * dt / (dx * dx);
    tau = 3.0 * nu_lbm + 0.5;
  }
  const double dm = rho_p * (dx * dx * dx);
  const double df = dm * dx / (dt * dt);
  out[0] = tau;
  out[1] = nu_lbm;
  out[2] = dm;
  out[3] = df;
  out[4] = kBT_p / (df * dx);
  out[5] = FORCE_LIMIT / 1.0e12 / df;
}

// CellMechanics::calculate_* (mechanics/cellMechanics.h:50-78) and the WBC
// constants (mechanics/wbcHighOrderModel.cpp:243-262).
void orc_material_scale(int model, int nfaces, const double* units, double dx, double dt, const double* mat,
                        double* k) {
  const double df = units[3], kBT = units[4];
  const double plc = 7.5e-9 / dx;
  const double eqL = 5e-7 / dx;
  const double nfs = 1280.0 / nfaces;
  k[0] = mat[0] * kBT / plc;
  k[1] = mat[1] * kBT / eqL;
  k[2] = mat[2] * nfs * kBT / eqL;
  k[3] = mat[3] * nfs * kBT / eqL;
  k[4] = mat[4] * dx / dt / df;
  k[5] = model == 2 ? mat[5] / df : 0.0;
  k[6] = model == 2 ? mat[6] / df : 0.0;
  k[7] = model == 2 ? mat[7] / dx : 0.0;
  k[8] = model == 2 ? mat[8] / dx : 0.0;
}

}  // extern "C"
