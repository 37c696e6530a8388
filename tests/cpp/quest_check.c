/* A C99 caller of the quest signed-distance C interface (include/gsq_quest.h),
 * written as a caller of the reference's shroud layer would be
 * (quest/interface/c_fortran/wrapQUEST.h), running the reference's interface
 * known answers (quest/tests/quest_signed_distance_interface.cpp): init fails
 * on an empty or missing file name (:337-349); an open planar mesh read from
 * an STL file gives phi = z on a 16^3 grid over [-4, 4]^3 to within 4 ulp
 * (EXPECT_DOUBLE_EQ, :186-242), with closest point (x, y, 0) and normal
 * (0, 0, 1); the mesh bounds are the nodes' (:372-404); finalize leaves the
 * query uninitialized; a second init as a closed, unsigned surface gives |z|.
 * Usage: quest_check <scratch STL path> [misuse 0-7]; with a misuse case it
 * prints "before" after init and then misuses the interface, which aborts.
 * Prints OK and exits 0 on success. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "gsq_quest.h"

static int failures = 0;

#define CHECK(cond, ...)              \
  do                                  \
  {                                   \
    if(!(cond))                       \
    {                                 \
      if(failures++ < 10)             \
      {                               \
        printf("FAILED %s: ", #cond); \
        printf(__VA_ARGS__);          \
        printf("\n");                 \
      }                               \
    }                                 \
  } while(0)

/* EXPECT_DOUBLE_EQ: within 4 units in the last place */
static int ulp_eq(double a, double b)
{
  if(a == b) return 1;
  if(isnan(a) || isnan(b) || (a < 0) != (b < 0)) return 0;
  int64_t ia, ib;
  memcpy(&ia, &a, 8);
  memcpy(&ib, &b, 8);
  const int64_t d = ia > ib ? ia - ib : ib - ia;
  return d <= 4;
}

/* the square [-5, 5]^2 in the plane z = 0 as four triangles around the
 * origin, counter-clockwise seen from +z (normal +z) */
static int write_plane(const char* path)
{
  static const double c[4][2] = {{5, -5}, {5, 5}, {-5, 5}, {-5, -5}};
  FILE* f = fopen(path, "w");
  if(!f) return 0;
  fprintf(f, "solid plane\n");
  for(int k = 0; k < 4; ++k)
  {
    const double* a = c[k];
    const double* b = c[(k + 1) % 4];
    fprintf(f, " facet normal 0.0 0.0 1.0\n  outer loop\n");
    fprintf(f, "   vertex %.1f %.1f 0.0\n   vertex %.1f %.1f 0.0\n   vertex 0.0 0.0 0.0\n", a[0], a[1], b[0], b[1]);
    fprintf(f, "  endloop\n endfacet\n");
  }
  fprintf(f, "endsolid plane\n");
  return fclose(f) == 0;
}

int main(int argc, char** argv)
{
  if(argc < 2) return 2;
  const char* file = argv[1];

  CHECK(QUEST_signed_distance_init_serial("") != 0, "init with an empty name");
  CHECK(QUEST_signed_distance_init_serial("badfile.stl") != 0, "init with a missing file");
  CHECK(!QUEST_signed_distance_initialized(), "initialized after failed inits");
  CHECK(write_plane(file), "cannot write %s", file);

  QUEST_signed_distance_set_dimension(3);
  QUEST_signed_distance_set_closed_surface(false);
  QUEST_signed_distance_set_execution_space(QUEST_SignedDistExec_GPU);
  CHECK(QUEST_signed_distance_init_serial(file) == 0, "init: %s", gsq_last_error());
  CHECK(QUEST_signed_distance_initialized(), "not initialized");
  if(failures)
  {
    printf("%d failures\n", failures);
    return 1;
  }
  if(argc > 2)
  {
    /* one misuse after init, which must abort the process as the reference's
     * death tests expect (quest_signed_distance_interface.cpp:245-335) */
    double lo[3];
    printf("before\n");
    fflush(stdout);
    switch(argv[2][0])
    {
    case '0': QUEST_signed_distance_set_closed_surface(true); break;
    case '1': QUEST_signed_distance_set_dimension(3); break;
    case '2': QUEST_signed_distance_set_verbose(true); break;
    case '3': QUEST_signed_distance_set_execution_space(QUEST_SignedDistExec_CPU); break;
    case '4': QUEST_signed_distance_get_mesh_bounds(NULL, lo); break;
    case '5': QUEST_signed_distance_set_compute_signs(false); break;
    case '6': QUEST_signed_distance_use_shared_memory(false); break;
    case '7': QUEST_signed_distance_set_allocator(0); break;
    default: break;
    }
    printf("after\n");
    return 3;
  }

  const int N = 16;
  for(int i = 0; i < N; ++i)
    for(int j = 0; j < N; ++j)
      for(int k = 0; k < N; ++k)
      {
        /* the uniform mesh's nodes: lo + i (hi - lo) / (N - 1) */
        const double x = -4.0 + i * (8.0 / (N - 1)), y = -4.0 + j * (8.0 / (N - 1)), z = -4.0 + k * (8.0 / (N - 1));
        const double phi = QUEST_signed_distance_evaluate_0(x, y, z);
        CHECK(ulp_eq(phi, z), "phi(%g, %g, %g) = %.17g", x, y, z, phi);
        double cx, cy, cz, nx, ny, nz;
        const double phi1 = QUEST_signed_distance_evaluate_1(x, y, z, &cx, &cy, &cz, &nx, &ny, &nz);
        CHECK(phi1 == phi, "evaluate_1 %.17g vs evaluate_0 %.17g", phi1, phi);
        CHECK(fabs(cx - x) <= 1e-12 && fabs(cy - y) <= 1e-12 && fabs(cz) <= 1e-12, "closest (%g %g %g)", cx, cy,
              cz);
        CHECK(fabs(nx) <= 1e-12 && fabs(ny) <= 1e-12 && fabs(nz - 1.0) <= 1e-12, "normal (%g %g %g)", nx, ny, nz);
      }

  double lo[3], hi[3];
  QUEST_signed_distance_get_mesh_bounds(lo, hi);
  CHECK(lo[0] == -5.0 && lo[1] == -5.0 && lo[2] == 0.0, "lo (%g %g %g)", lo[0], lo[1], lo[2]);
  CHECK(hi[0] == 5.0 && hi[1] == 5.0 && hi[2] == 0.0, "hi (%g %g %g)", hi[0], hi[1], hi[2]);

  /* a second init while initialized fails and keeps the query */
  CHECK(QUEST_signed_distance_init_serial(file) != 0, "second init succeeded");
  CHECK(QUEST_signed_distance_initialized(), "second init dropped the query");

  QUEST_signed_distance_finalize();
  CHECK(!QUEST_signed_distance_initialized(), "initialized after finalize");

  /* unsigned, through the Fortran-style entry with a blank-padded name */
  QUEST_signed_distance_set_closed_surface(true);
  QUEST_signed_distance_set_compute_signs(false);
  char padded[1024];
  const size_t len = strlen(file);
  if(len + 8 < sizeof(padded))
  {
    memcpy(padded, file, len);
    memset(padded + len, ' ', 8);
    CHECK(QUEST_signed_distance_init_serial_bufferify(padded, (int)(len + 8)) == 0, "bufferify init: %s",
          gsq_last_error());
    for(int k = 0; k < N; ++k)
    {
      const double z = -4.0 + k * (8.0 / (N - 1));
      const double phi = QUEST_signed_distance_evaluate_0(0.25, -1.5, z);
      CHECK(ulp_eq(phi, fabs(z)), "unsigned phi(z = %g) = %.17g", z, phi);
    }
    QUEST_signed_distance_finalize();
  }
  CHECK(!QUEST_signed_distance_initialized(), "initialized after the last finalize");

  if(failures)
  {
    printf("%d failures\n", failures);
    return 1;
  }
  printf("OK\n");
  return 0;
}
