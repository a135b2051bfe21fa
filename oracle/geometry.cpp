// Cell geometry of the FP64 CPU oracle (test infrastructure only): the mesh
// generators, loadParticles' placement and the seeded packer, restated
// without any code of the product library so that the product's meshes and
// placements can be checked bit for bit.  Built into liboracle.so with
// -ffp-contract=off; the product compiles its host geometry the same way,
// so on one machine the two give identical doubles.
//
//   icosphere          constructSphereIcosahedron, helper/meshGeneratingFunctions.hh:31-151
//   RBC template       constructRBCFromSphere + spherePointToRBCPoint, :153-168, :213-241
//   ellipsoid template constructEllipsoidFromSphere + spherePointToEllipsoidPoint, :170-183, :244-271
//   placement          rotateTriangularMeshXYZ, meshRotation and the starting-point
//                      offset of io/readPositionsBloodCells.cpp:39-124, 290-361
//   .pos conversion    getReadPositionsBloodCellsVector, io/readPositionsBloodCells.cpp:186-285
//
// Conventions that the reference leaves to Palabos (not in its tree) and
// that this oracle fixes the way the product documents them:
//   - vertex numbering: corners merged by bit pattern, numbered by first
//     appearance in the refined triangle soup;
//   - TriangleSet::rotate(phi, theta, psi): Euler angles in the x-convention
//     (Goldstein's A = B(psi) C(theta) D(phi), applied as p' = A p);
//   - Palabos inflate() of the finished template: not applied.
// The seeded packer and the antipodal inner-link pairs have no reference
// counterpart (tools/packCells is a different, force-based program); they
// are the project's own algorithms, restated here so that the synthetic
// workloads can be built without the product library.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#include "oracle.h"

namespace {

struct P3 {
  double c[3];
};

double norm3(const P3& p) {
  double s = 0.0;
  s += p.c[0] * p.c[0];
  s += p.c[1] * p.c[1];
  s += p.c[2] * p.c[2];
  return std::sqrt(s);
}

// the refined icosahedron as a triangle soup on the unit sphere
std::vector<P3> sphere_soup(int min_triangles) {
  const double t = -0.8506508084, o = -0.5257311121;
  const double ico[12][3] = {{t, o, 0},  {-t, o, 0}, {-t, -o, 0}, {t, -o, 0}, {o, 0, t},  {o, 0, -t},
                             {-o, 0, -t}, {-o, 0, t}, {0, t, o},   {0, -t, o}, {0, -t, -o}, {0, t, -o}};
  // faces as 1-based corners, in the order the reference pushes them
  const int face[20][3] = {{5, 8, 9},  {5, 10, 8}, {6, 12, 7}, {6, 7, 11}, {1, 4, 5},  {1, 6, 4},  {3, 2, 8},
                           {3, 7, 2},  {9, 12, 1}, {9, 2, 12}, {10, 4, 11}, {10, 11, 3}, {9, 1, 5},  {12, 6, 1},
                           {5, 4, 10}, {6, 11, 4}, {8, 2, 9},  {7, 12, 2}, {8, 10, 3}, {7, 3, 11}};
  std::vector<P3> soup;  // 3 corners per triangle
  for (const auto& f : face)
    for (int k = 0; k < 3; ++k) soup.push_back(P3{{ico[f[k] - 1][0], ico[f[k] - 1][1], ico[f[k] - 1][2]}});
  auto midpoint = [](const P3& a, const P3& b) {
    P3 m{{(a.c[0] + b.c[0]) * 0.5, (a.c[1] + b.c[1]) * 0.5, (a.c[2] + b.c[2]) * 0.5}};
    const double l = norm3(m);
    for (double& x : m.c) x = x / l;
    return m;
  };
  for (;;) {
    const size_t ntri = soup.size() / 3;
    if ((long)ntri >= (long)min_triangles) break;
    for (size_t i = 0; i < ntri; ++i) {
      const P3 a = soup[3 * i], b = soup[3 * i + 1], c = soup[3 * i + 2];
      const P3 d = midpoint(a, b), e = midpoint(b, c), f = midpoint(c, a);
      soup[3 * i] = d;
      soup[3 * i + 1] = e;
      soup[3 * i + 2] = f;
      const P3 add[9] = {a, d, f, d, b, e, f, e, c};
      for (const P3& q : add) soup.push_back(q);
    }
  }
  return soup;
}

struct MeshOut {
  std::vector<P3> v;
  std::vector<int> t;  // 3 per face
};

MeshOut merge(const std::vector<P3>& soup) {
  MeshOut m;
  std::map<std::vector<uint64_t>, int> seen;
  for (const P3& p : soup) {
    std::vector<uint64_t> key(3);
    for (int a = 0; a < 3; ++a) std::memcpy(&key[a], &p.c[a], sizeof(double));
    auto it = seen.find(key);
    int id;
    if (it == seen.end()) {
      id = (int)m.v.size();
      seen.emplace(key, id);
      m.v.push_back(p);
    } else {
      id = it->second;
    }
    m.t.push_back(id);
  }
  return m;
}

// TriangleSet::rotate(phi, theta, psi) in the x-convention, p' = A p
struct Rot {
  double a[3][3];
  Rot(double phi, double theta, double psi) {
    const double cf = std::cos(phi), sf = std::sin(phi);
    const double ct = std::cos(theta), st = std::sin(theta);
    const double cp = std::cos(psi), sp = std::sin(psi);
    a[0][0] = cp * cf - ct * sf * sp;
    a[0][1] = cp * sf + ct * cf * sp;
    a[0][2] = sp * st;
    a[1][0] = -sp * cf - ct * sf * cp;
    a[1][1] = -sp * sf + ct * cf * cp;
    a[1][2] = cp * st;
    a[2][0] = st * sf;
    a[2][1] = -st * cf;
    a[2][2] = ct;
  }
  P3 apply(const P3& p) const {
    P3 r;
    for (int i = 0; i < 3; ++i) r.c[i] = a[i][0] * p.c[0] + a[i][1] * p.c[1] + a[i][2] * p.c[2];
    return r;
  }
};

int sign_of(double v) { return (0.0 < v) - (v < 0.0); }

int export_mesh(const MeshOut& m, double* xyz, int max_nv, int* tris, int max_nf, int* nv, int* nf) {
  const int V = (int)m.v.size(), F = (int)m.t.size() / 3;
  *nv = V;
  *nf = F;
  if (V > max_nv || F > max_nf) return -1;
  for (int i = 0; i < V; ++i)
    for (int a = 0; a < 3; ++a) xyz[3 * i + a] = m.v[i].c[a];
  for (int k = 0; k < 3 * F; ++k) tris[k] = m.t[k];
  return 0;
}

// loadParticles' placement of one cell: centre the template on its bounding
// box, meshRotation, then the starting point
void place_one(const double* rest, int nv, const double start[3], const double ang[3], double* out) {
  std::vector<double> v(rest, rest + 3 * nv);
  double lo[3], hi[3];
  auto bbox = [&]() {
    for (int a = 0; a < 3; ++a) {
      lo[a] = 1e300;
      hi[a] = -1e300;
    }
    for (int i = 0; i < nv; ++i)
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], v[3 * i + a]);
        hi[a] = std::max(hi[a], v[3 * i + a]);
      }
  };
  bbox();
  double shift[3];
  for (int a = 0; a < 3; ++a) shift[a] = -(lo[a] + hi[a]) / 2.0;
  for (int i = 0; i < nv; ++i)
    for (int a = 0; a < 3; ++a) v[3 * i + a] = v[3 * i + a] + shift[a];
  bbox();
  double mc[3];
  for (int a = 0; a < 3; ++a) mc[a] = (hi[a] + lo[a]) * 0.5;
  // rotateTriangularMeshXYZ: x, then y (c = Ry * Rx), then z (Rz * c), the
  // factors stored column-first as in the reference
  double ra[3][3] = {{1.0, 0.0, 0.0},
                     {0.0, std::cos(ang[0]), std::sin(ang[0])},
                     {0.0, -std::sin(ang[0]), std::cos(ang[0])}};
  double rb[3][3] = {{std::cos(ang[1]), 0.0, -std::sin(ang[1])},
                     {0.0, 1.0, 0.0},
                     {std::sin(ang[1]), 0.0, std::cos(ang[1])}};
  double rc[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      rc[i][j] = 0.0;
      for (int k = 0; k < 3; ++k) rc[i][j] += ra[k][j] * rb[i][k];
    }
  const double rz[3][3] = {{std::cos(ang[2]), std::sin(ang[2]), 0.0},
                           {-std::sin(ang[2]), std::cos(ang[2]), 0.0},
                           {0.0, 0.0, 1.0}};
  double m[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      m[i][j] = 0.0;
      for (int k = 0; k < 3; ++k) m[i][j] += rc[k][j] * rz[i][k];
    }
  for (int i = 0; i < nv; ++i) {
    double x[3];
    for (int a = 0; a < 3; ++a) x[a] = v[3 * i + a] + (-1.0 * mc[a]);
    for (int a = 0; a < 3; ++a) {
      double r = 0.0;
      for (int b = 0; b < 3; ++b) r += m[a][b] * x[b];
      out[3 * i + a] = start[a] + (r + mc[a]);
    }
  }
}

// ---------------------------------------------------------------------------
// Seeded packer (the project's own algorithm): random sequential addition of
// the largest shapes first, then a Monte-Carlo relaxation of overlaps.  The
// occupancy of a placed cell is its vertices' nearest nodes plus the nodes
// inside its surface (scanline parity along z per (x, y) column).

struct Rng {
  uint64_t s;
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double a = std::max(u01(), 1e-300);
    const double b = u01();
    return std::sqrt(-2.0 * std::log(a)) * std::cos(2 * M_PI * b);
  }
  // a uniformly distributed rotation, as reference-convention angles (the
  // reference rotates by the negated .pos angles)
  void rotation(double* ang) {
    const double x = (2 * u01() - 1) * M_PI;
    const double y = std::asin(2 * u01() - 1);
    const double z = (2 * u01() - 1) * M_PI;
    ang[0] = -x;
    ang[1] = -y;
    ang[2] = -z;
  }
};

struct Lattice {
  int n[3];
  int per[3];
  // wrap on periodic axes; false off a closed axis
  bool wrap(long* q) const {
    for (int a = 0; a < 3; ++a)
      if (q[a] < 0 || q[a] >= n[a]) {
        if (!per[a]) return false;
        q[a] = ((q[a] % n[a]) + n[a]) % n[a];
      }
    return true;
  }
  long index(const long* q) const { return q[0] + (long)n[0] * (q[1] + (long)n[1] * q[2]); }
};

bool covered_nodes(const Lattice& lat, const std::vector<double>& xyz, const int* tris, int nf, std::vector<long>& out,
                   std::vector<std::pair<long, double>>& cross) {
  out.clear();
  cross.clear();
  const int nv = (int)(xyz.size() / 3);
  for (int i = 0; i < nv; ++i) {
    long q[3];
    for (int a = 0; a < 3; ++a) q[a] = (long)std::floor(xyz[3 * i + a] + 0.5);
    if (!lat.wrap(q)) return false;
    out.push_back(lat.index(q));
  }
  const long K = 1 << 20;
  for (int f = 0; f < nf; ++f) {
    const double* A = &xyz[3 * tris[3 * f]];
    const double* B = &xyz[3 * tris[3 * f + 1]];
    const double* C = &xyz[3 * tris[3 * f + 2]];
    const double det = (B[0] - A[0]) * (C[1] - A[1]) - (C[0] - A[0]) * (B[1] - A[1]);
    if (std::fabs(det) < 1e-14) continue;
    const long x0 = (long)std::ceil(std::min({A[0], B[0], C[0]})), x1 = (long)std::floor(std::max({A[0], B[0], C[0]}));
    const long y0 = (long)std::ceil(std::min({A[1], B[1], C[1]})), y1 = (long)std::floor(std::max({A[1], B[1], C[1]}));
    for (long X = x0; X <= x1; ++X)
      for (long Y = y0; Y <= y1; ++Y) {
        // a ray along z through a point nudged off the node lattice
        const double px = X + 1e-7, py = Y + 2.3e-7;
        const double u = ((px - A[0]) * (C[1] - A[1]) - (C[0] - A[0]) * (py - A[1])) / det;
        const double w = ((B[0] - A[0]) * (py - A[1]) - (px - A[0]) * (B[1] - A[1])) / det;
        if (u < 0 || w < 0 || u + w > 1) continue;
        cross.push_back({(X + K) * (2 * K) + (Y + K), A[2] + u * (B[2] - A[2]) + w * (C[2] - A[2])});
      }
  }
  std::sort(cross.begin(), cross.end());
  size_t k = 0;
  while (k + 1 < cross.size()) {
    size_t e = k;
    while (e < cross.size() && cross[e].first == cross[k].first) ++e;
    const long X = cross[k].first / (2 * K) - K, Y = cross[k].first % (2 * K) - K;
    for (size_t j = k; j + 1 < e; j += 2)
      for (long Z = (long)std::ceil(cross[j].second); Z <= (long)std::floor(cross[j + 1].second); ++Z) {
        long q[3] = {X, Y, Z};
        if (!lat.wrap(q)) return false;
        out.push_back(lat.index(q));
      }
    k = e;
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return true;
}

struct Placed {
  int type;
  double c[3], a[3];
  std::vector<long> nodes;
};

}  // namespace

extern "C" {

int orc_mesh_icosphere(int min_triangles, double radius, double* xyz, int max_nv, int* tris, int max_nf, int* nv,
                       int* nf) {
  MeshOut m = merge(sphere_soup(min_triangles));
  for (P3& p : m.v)
    for (double& x : p.c) x = x * radius;
  return export_mesh(m, xyz, max_nv, tris, max_nf, nv, nf);
}

int orc_mesh_rbc(int min_triangles, double radius, double* xyz, int max_nv, int* tris, int max_nf, int* nv, int* nf) {
  MeshOut m = merge(sphere_soup(min_triangles));
  const Rot R(M_PI / 2.0, M_PI / 2.0, 0.0);
  const double C0 = 0.054322, C2 = 1.001279, C4 = -0.561381;
  for (P3& p : m.v) {
    P3 s = R.apply(p);
    double r2 = s.c[0] * s.c[0] + s.c[1] * s.c[1];
    const int sg = sign_of(s.c[2]);
    if (1 - r2 < 0) r2 = 1;
    s.c[2] = sg * std::sqrt(1 - r2) * (C0 + C2 * r2 + C4 * r2 * r2);
    for (double& x : s.c) x = x * radius;
    p = R.apply(s);
  }
  return export_mesh(m, xyz, max_nv, tris, max_nf, nv, nf);
}

int orc_mesh_ellipsoid(int min_triangles, double radius, double aspect, double* xyz, int max_nv, int* tris,
                       int max_nf, int* nv, int* nf) {
  MeshOut m = merge(sphere_soup(min_triangles));
  const Rot R(M_PI / 2.0, M_PI / 2.0, 0.0);
  for (P3& p : m.v) {
    P3 s = R.apply(p);
    double r2 = s.c[0] * s.c[0] + s.c[1] * s.c[1];
    const int sg = sign_of(s.c[2]);
    if (1 - r2 < 0) r2 = 1;
    s.c[0] = s.c[0] * radius;
    s.c[1] = s.c[1] * radius;
    s.c[2] = sg * aspect * radius * std::sqrt(1 - r2);
    p = R.apply(s);
  }
  return export_mesh(m, xyz, max_nv, tris, max_nf, nv, nf);
}

// for each vertex i, the first j > i with |x_i + x_j| < 1e-9 * max(1, max |x|)
int orc_mesh_antipodal_pairs(const double* xyz, int nv, int* pairs, int max_pairs) {
  double big = 0;
  for (int i = 0; i < nv; ++i) {
    P3 p{{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}};
    big = std::max(big, norm3(p));
  }
  const double tol = 1e-9 * std::max(big, 1.0);
  int n = 0;
  for (int i = 0; i < nv; ++i)
    for (int j = i + 1; j < nv; ++j) {
      P3 s{{xyz[3 * i] + xyz[3 * j], xyz[3 * i + 1] + xyz[3 * j + 1], xyz[3 * i + 2] + xyz[3 * j + 2]}};
      if (norm3(s) < tol) {
        if (n >= max_pairs) return -1;
        pairs[2 * n] = i;
        pairs[2 * n + 1] = j;
        ++n;
        break;
      }
    }
  return n;
}

void orc_place_cells(const double* rest, int nv, int n, const double* centres, const double* angles, double* out) {
  for (int c = 0; c < n; ++c) place_one(rest, nv, centres + 3 * c, angles + 3 * c, out + (size_t)3 * nv * c);
}

void orc_pos_to_lattice(int n, const double* pos_um, const double* angles_deg, double dx, double* centres,
                        double* angles) {
  const double to_lu = 1e-6 / dx;
  for (int c = 0; c < n; ++c)
    for (int a = 0; a < 3; ++a) {
      centres[3 * c + a] = pos_um[3 * c + a] * to_lu + 0.0;
      double r = angles_deg[3 * c + a] * (M_PI / 180.0);
      angles[3 * c + a] = r * -1.0;
    }
}

int orc_pack_cells(int nx, int ny, int nz, const int* periodic, const uint8_t* solid, int ntypes,
                   const double* const* rest, const int* nvs, const int* const* tris, const int* nfs,
                   const int* counts, double margin, unsigned long long seed, int max_attempts, double* centres,
                   double* angles, int* types) {
  Lattice lat{{nx, ny, nz}, {periodic[0], periodic[1], periodic[2]}};
  const long N = (long)nx * ny * nz;
  std::vector<uint8_t> forbidden(N, 0);
  std::vector<uint16_t> count(N, 0);
  if (solid) {
    const int r = (int)std::ceil(std::max(margin, 0.0));
    for (long Z = 0; Z < nz; ++Z)
      for (long Y = 0; Y < ny; ++Y)
        for (long X = 0; X < nx; ++X) {
          if (!solid[X + nx * (Y + (long)ny * Z)]) continue;
          for (int dz = -r; dz <= r; ++dz)
            for (int dy = -r; dy <= r; ++dy)
              for (int dx = -r; dx <= r; ++dx) {
                if (dx * dx + dy * dy + dz * dz > margin * margin + 1e-9) continue;
                long q[3] = {X + dx, Y + dy, Z + dz};
                if (lat.wrap(q)) forbidden[lat.index(q)] = 1;
              }
        }
  }
  // largest shapes (by the farthest vertex from the origin) first, ties in type order
  std::vector<double> reach(ntypes, 0.0);
  for (int t = 0; t < ntypes; ++t)
    for (int i = 0; i < nvs[t]; ++i) {
      const double* p = rest[t] + 3 * i;
      reach[t] = std::max(reach[t], std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
    }
  std::vector<int> order(ntypes);
  for (int t = 0; t < ntypes; ++t) order[t] = t;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reach[a] > reach[b]; });

  Rng rng{seed};
  std::vector<double> xyz;
  std::vector<std::pair<long, double>> cross;
  std::vector<Placed> cells;
  // overlap count of a candidate, or -1 when it leaves a closed axis or
  // enters a forbidden node
  auto score = [&](int t, const double* c, const double* a, std::vector<long>& nodes) -> long {
    xyz.assign((size_t)3 * nvs[t], 0.0);
    place_one(rest[t], nvs[t], c, a, xyz.data());
    if (!covered_nodes(lat, xyz, tris[t], nfs[t], nodes, cross)) return -1;
    long ov = 0;
    for (long q : nodes) {
      if (forbidden[q]) return -1;
      ov += count[q];
    }
    return ov;
  };
  const int tries = std::max(1, std::min(max_attempts, 300));
  for (int t : order)
    for (int c = 0; c < counts[t]; ++c) {
      Placed best;
      long best_ov = -1;
      for (int k = 0; k < tries; ++k) {
        Placed p;
        p.type = t;
        for (int a = 0; a < 3; ++a) p.c[a] = rng.u01() * lat.n[a] - 0.5;
        rng.rotation(p.a);
        const long ov = score(t, p.c, p.a, p.nodes);
        if (ov < 0) continue;
        if (best_ov < 0 || ov < best_ov) {
          best = p;
          best_ov = ov;
        }
        if (ov == 0) break;
      }
      if (best_ov < 0) return (int)cells.size();
      for (long q : best.nodes) count[q]++;
      cells.push_back(best);
    }
  auto excess = [&](const Placed& p) {
    long e = 0;
    for (long q : p.nodes) e += count[q] - 1;
    return e;
  };
  const long budget = (long)std::max(1, max_attempts) * (long)std::max<size_t>(cells.size(), 1);
  long used = 0;
  std::vector<int> overlapping;
  while (used < budget) {
    overlapping.clear();
    for (int i = 0; i < (int)cells.size(); ++i)
      if (excess(cells[i]) > 0) overlapping.push_back(i);
    if (overlapping.empty()) break;
    // Fisher-Yates from the back
    for (int k = (int)overlapping.size() - 1; k > 0; --k) std::swap(overlapping[k], overlapping[rng.next() % (k + 1)]);
    for (int i : overlapping) {
      Placed& p = cells[i];
      long cur = excess(p);
      if (cur == 0) continue;
      for (long q : p.nodes) count[q]--;
      for (int k = 0; k < 8 && cur > 0; ++k, ++used) {
        Placed cand = p;
        const double step = 0.5 + 1.5 * rng.u01();
        for (int a = 0; a < 3; ++a) cand.c[a] = p.c[a] + step * rng.normal();
        if (rng.u01() < 0.2) {
          rng.rotation(cand.a);
        } else {
          for (int a = 0; a < 3; ++a) cand.a[a] = p.a[a] + 0.3 * rng.normal();
        }
        const long ov = score(p.type, cand.c, cand.a, cand.nodes);
        if (ov >= 0 && ov <= cur) {
          p = cand;
          cur = ov;
        }
      }
      for (long q : p.nodes) count[q]++;
    }
  }
  int placed = 0;
  for (const Placed& p : cells) {
    if (excess(p) > 0) continue;
    for (int a = 0; a < 3; ++a) {
      double c = p.c[a];
      if (lat.per[a]) c = std::fmod(std::fmod(c + 0.5, (double)lat.n[a]) + lat.n[a], (double)lat.n[a]) - 0.5;
      centres[3 * placed + a] = c;
      angles[3 * placed + a] = p.a[a];
    }
    types[placed] = p.type;
    ++placed;
  }
  return placed;
}

}  // extern "C"
