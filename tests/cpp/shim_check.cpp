// C++ caller of the gsq.hpp shim, written like the reference's own tests:
// the 3x3x3 uniform-mesh known answers of spin/tests/spin_bvh.cpp:279-406 and
// 519-648, and the exact plane of
// quest/tests/quest_signed_distance_interface.cpp:186-242.
#include <cmath>
#include <cstdio>
#include <set>

#include "gsq.hpp"

static int failures = 0;
#define EXPECT(c)                                               \
  do                                                            \
  {                                                             \
    if(!(c))                                                    \
    {                                                           \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
      ++failures;                                               \
    }                                                           \
  } while(0)

int main()
{
  // 27 cells of a 3x3x3 uniform mesh over [0,3]^3, cell i fastest
  std::vector<gsq::BoundingBox> cells;
  for(int k = 0; k < 3; ++k)
    for(int j = 0; j < 3; ++j)
      for(int i = 0; i < 3; ++i)
        cells.push_back({{double(i), double(j), double(k)}, {double(i + 1), double(j + 1), double(k + 1)}});
  gsq::spin::BVH<3, double> bvh;
  bvh.setScaleFactor(1.0);
  EXPECT(bvh.initialize(cells.data(), (int32_t)cells.size()) == gsq::spin::BVH_BUILD_OK);
  const gsq::BoundingBox b = bvh.getBounds();
  for(int d = 0; d < 3; ++d) EXPECT(std::fabs(b.min[d]) < 1e-12 && std::fabs(b.max[d] - 3.0) < 1e-12);

  gsq::BoundingBox q[2] = {{{-1, -1, -1}, {2.5, 2.5, 1.5}}, {{-1, -1, -1}, {-0.5, -0.5, -0.5}}};
  gsq::Candidates c;
  bvh.findBoundingBoxes(c, 2, q);
  EXPECT(c.counts[0] == 18 && c.counts[1] == 0);
  std::set<int> hit(c.candidates.begin() + c.offsets[0], c.candidates.begin() + c.offsets[0] + c.counts[0]);
  for(int i = 0; i < 18; ++i) EXPECT(hit.count(i) == 1);

  const double up[3] = {1, 1, 1}, down[3] = {-1, -1, -1};
  gsq::Ray rays[2] = {gsq::Ray({{-1, -1, -1}}, up), gsq::Ray({{-1, -1, -1}}, down)};
  bvh.findRays(c, 2, rays);
  EXPECT(c.counts[0] == 15 && c.counts[1] == 0);

  gsq::quest::SurfaceMesh plane;
  plane.x = {-5, 5, 0, 5, -5};
  plane.y = {-5, -5, 0, 5, 5};
  plane.z = {0, 0, 0, 0, 0};
  plane.cells = {0, 1, 2, 1, 3, 2, 3, 4, 2, 4, 0, 2};
  for(int precision : {GSQ_PRECISION_FP64, GSQ_PRECISION_MIXED})
  {
    gsq::quest::SignedDistance<3> sd(plane, /*isWatertight=*/false, true, precision);
    for(int k = 0; k < 16; ++k)
      for(int j = 0; j < 16; ++j)
        for(int i = 0; i < 16; ++i)
        {
          const gsq::Point p {{-4.0 + i * 8.0 / 15, -4.0 + j * 8.0 / 15, -4.0 + k * 8.0 / 15}};
          const double d = sd.computeDistance(p);
          EXPECT(std::fabs(d - p.x[2]) <= 4 * 2.220446049250313e-16 * std::fabs(p.x[2]));
        }
  }
  // STL round trip: the plane's four triangles as an ASCII file, read back
  // through the reader and evaluated like the mesh above
  {
    const char* path = "shim_check_plane.stl";
    FILE* f = std::fopen(path, "w");
    EXPECT(f != nullptr);
    std::fprintf(f, "solid plane\n");
    for(size_t t = 0; t < plane.cells.size(); t += 3)
    {
      std::fprintf(f, "facet normal 0 0 1\nouter loop\n");
      for(int k = 0; k < 3; ++k)
      {
        const int v = plane.cells[t + k];
        std::fprintf(f, "vertex %.17g %.17g %.17g\n", plane.x[v], plane.y[v], plane.z[v]);
      }
      std::fprintf(f, "endloop\nendfacet\n");
    }
    std::fprintf(f, "endsolid plane\n");
    std::fclose(f);
    gsq::quest::STLReader reader;
    reader.setFileName(path);
    EXPECT(reader.read() == 0);
    gsq::quest::SurfaceMesh m;
    reader.getMesh(m);
    EXPECT(m.x.size() == 12 && m.numCells() == 4);
    gsq::quest::SignedDistance<3> sd(m, false);
    const gsq::Point p {{0.5, -1.25, 2.0}};
    EXPECT(std::fabs(sd.computeDistance(p) - 2.0) <= 1e-15);
    std::remove(path);
  }

  // the C-style interface with a mesh (quest_signed_distance_interface.cpp:
  // 372-404 bounds, 186-242 plane values): init, evaluate in the three
  // forms, bounds, finalize
  {
    EXPECT(!gsq::quest::signed_distance_initialized());
    gsq::quest::signed_distance_set_closed_surface(false);
    gsq::quest::signed_distance_set_execution_space(gsq::quest::SignedDistExec::GPU);
    EXPECT(gsq::quest::signed_distance_init(&plane) == 0);
    EXPECT(gsq::quest::signed_distance_initialized());
    double xs[3] = {0.5, -3.0, 4.0}, ys[3] = {-1.25, 2.0, 4.0}, zs[3] = {2.0, -0.75, 3.5}, phi[3];
    gsq::quest::signed_distance_evaluate(xs, ys, zs, 3, phi);
    for(int i = 0; i < 3; ++i)
    {
      EXPECT(std::fabs(phi[i] - zs[i]) <= 4 * 2.220446049250313e-16 * std::fabs(zs[i]));
      EXPECT(gsq::quest::signed_distance_evaluate(xs[i], ys[i], zs[i]) == phi[i]);
      double cx, cy, cz, nx, ny, nz;
      EXPECT(gsq::quest::signed_distance_evaluate(xs[i], ys[i], zs[i], cx, cy, cz, nx, ny, nz) == phi[i]);
      EXPECT(std::fabs(cx - xs[i]) <= 1e-12 && std::fabs(cy - ys[i]) <= 1e-12 && std::fabs(cz) <= 1e-12);
      EXPECT(std::fabs(nz - 1.0) <= 1e-12);
    }
    double lo[3], hi[3];
    gsq::quest::signed_distance_get_mesh_bounds(lo, hi);
    EXPECT(lo[0] == -5 && lo[1] == -5 && lo[2] == 0 && hi[0] == 5 && hi[1] == 5 && hi[2] == 0);
    gsq::quest::signed_distance_finalize();
    EXPECT(!gsq::quest::signed_distance_initialized());
  }

  // closest object point: the 27 cell corners (0..3)^3 minus one
  {
    std::vector<gsq::Point> pts;
    for(int k = 0; k < 4; ++k)
      for(int j = 0; j < 4; ++j)
        for(int i = 0; i < 4; ++i) pts.push_back({{double(i), double(j), double(k)}});
    gsq::quest::ClosestPoint cp((int32_t)pts.size(), pts.data());
    const gsq::Point qs[2] = {{{1.1, 2.2, 2.9}}, {{10.0, 10.0, 10.0}}};
    int32_t idx[2], dom[2];
    gsq::Point pos[2];
    double dist[2];
    cp.computeClosestPoints(2, qs, idx, dom, pos, dist);
    EXPECT(idx[0] == 1 + 4 * 2 + 16 * 3 && dom[0] == 0);
    EXPECT(pos[0].x[0] == 1.0 && pos[0].x[1] == 2.0 && pos[0].x[2] == 3.0);
    cp.setDistanceThreshold(1.0);
    cp.computeClosestPoints(2, qs, idx, dom, pos, dist);
    EXPECT(idx[0] >= 0 && idx[1] == -1 && dist[1] != dist[1]);
  }

  std::printf("%s (%d failures)\n", failures ? "FAIL" : "OK", failures);
  return failures ? 1 : 0;
}
