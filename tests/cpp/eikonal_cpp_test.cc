// C++ drop-in check: the reference's own test programs (src/test/3d/3D-small.cc,
// 3D-basic.cc, 3D-converge.cc, 3D-sanity.cc, src/test/2d/2D-basic.cc,
// 2D-sanity.cc, 2D-converge.cc) restated against include/Eikonal.h, with a small
// assertion helper in place of gtest.  argv[1] is the directory holding the
// fixture meshes (sphere8.node/.ele, ..., sphere_74verts.ply, ...).
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "Eikonal.h"

static int g_fail = 0, g_checks = 0;
#define EXPECT(c)                                                         \
  do {                                                                    \
    ++g_checks;                                                           \
    if (!(c)) {                                                           \
      ++g_fail;                                                           \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);          \
    }                                                                     \
  } while (0)
#define EXPECT_NO_THROW(s)                                                \
  do {                                                                    \
    ++g_checks;                                                           \
    try {                                                                 \
      s;                                                                  \
    } catch (const std::exception& e) {                                   \
      ++g_fail;                                                           \
      std::printf("FAILED %s:%d: %s threw %s\n", __FILE__, __LINE__, #s, e.what()); \
    }                                                                     \
  } while (0)
#define EXPECT_THROW(s)                                                   \
  do {                                                                    \
    ++g_checks;                                                           \
    bool thrown = false;                                                  \
    try {                                                                 \
      s;                                                                  \
    } catch (const std::runtime_error&) {                                 \
      thrown = true;                                                      \
    }                                                                     \
    if (!thrown) {                                                        \
      ++g_fail;                                                           \
      std::printf("FAILED %s:%d: %s did not throw\n", __FILE__, __LINE__, #s); \
    }                                                                     \
  } while (0)

static std::string D;

// final result, or an empty vector when the solve failed (already reported)
static const std::vector<float>& fin(Eikonal& e) {
  static const std::vector<float> empty;
  return e.numIterations() ? e.getFinalResult() : empty;
}

static void small3d() {
  Eikonal data(false);
  data.filename_ = D + "sphere8";
  data.maxBlocks_ = 100;
  EXPECT_NO_THROW(data.solveEikonal());
  if (fin(data).empty()) return;
  EXPECT(fin(data)[0] == 0.f);
  for (size_t i = 1; i < fin(data).size(); i++)
    EXPECT(std::fabs(fin(data)[i] - 19.58f) <= 4 * 19.58f * 1.1920929e-7f);
  Eikonal d13(false);
  d13.filename_ = D + "sphere13";
  d13.maxBlocks_ = 100;
  EXPECT_NO_THROW(d13.solveEikonal());
  if (fin(d13).empty()) return;
  EXPECT(std::fabs(fin(d13)[0]) <= 1e-4f);
  for (size_t i = 1; i < fin(d13).size(); i++) EXPECT(std::fabs(fin(d13)[i] - 19.58f) <= 1e-4f);
}

static void basic3d() {
  Eikonal a(false);
  a.filename_ = D + "sphere334";
  EXPECT_NO_THROW(a.solveEikonal());
  for (float v : fin(a)) EXPECT(v < 100.f);
  Eikonal b(false);
  b.filename_ = D + "CubeMesh_size16";
  b.isStructured_ = true;
  EXPECT_NO_THROW(b.solveEikonal());
  for (float v : fin(b)) EXPECT(v < 100.f);
}

static void converge3d(bool structured) {
  Eikonal data(false);
  data.filename_ = D + (structured ? "CubeMesh_size16" : "sphere334");
  data.isStructured_ = structured;
  EXPECT_NO_THROW(data.solveEikonal());
  EXPECT(data.numIterations() > 2);
  for (size_t i = 2; i < data.numIterations(); i++)
    for (size_t j = 0; j < data.getResultAtIteration(i).size(); j++) {
      const float one = data.getResultAtIteration(i - 1)[j];
      const float zero = data.getResultAtIteration(i)[j];
      if (one == 0.) continue;
      EXPECT(zero <= one);
    }
}

static void sanity3d() {
  Eikonal data(false);
  data.filename_ = "notarealfile";
  EXPECT_THROW(data.solveEikonal());  // the reference exits with status 1
  Eikonal b(false);
  b.filename_ = D + "sphere334";
  EXPECT_NO_THROW(b.solveEikonal());
}

static void basic2d() {
  Eikonal a(true);
  a.filename_ = D + "sphere_74verts.ply";
  a.maxBlocks_ = 11;
  a.stopDistance_ = 700.f;
  EXPECT_NO_THROW(a.solveEikonal());
  for (float v : fin(a)) EXPECT(v < a.stopDistance_);
  Eikonal b(true);
  b.filename_ = D + "SquareMesh_size16.ply";
  b.squareLength_ = 16;
  b.squareWidth_ = 16;
  b.squareBlockLength_ = 4;
  b.squareBlockWidth_ = 4;
  b.stopDistance_ = 100.f;
  b.isStructured_ = true;
  EXPECT_NO_THROW(b.solveEikonal());
  for (float v : fin(b)) EXPECT(v < b.stopDistance_);
  EXPECT(b.maxBlocks_ == 16);  // overwritten with the tiling's block count
}

static void sanity_converge2d() {
  Eikonal bad(true);
  bad.filename_ = "notarealfile";
  EXPECT_THROW(bad.solveEikonal());
  Eikonal data(true);
  data.filename_ = D + "sphere_74verts.ply";
  data.maxBlocks_ = 1000;
  EXPECT_NO_THROW(data.solveEikonal());
  for (size_t i = 1; i < data.numIterations(); i++)
    for (size_t j = 0; j < fin(data).size(); j++)
      EXPECT(data.getResultAtIteration(i)[j] <= data.getResultAtIteration(i - 1)[j]);
}

static void seeds_and_speeds() {
  // initializeVertices before a mesh is an error; afterwards zeros are seeds
  Eikonal e(false);
  e.filename_ = D + "sphere334";
  EXPECT_THROW(e.initializeVertices(std::vector<float>(334, 1e9f)));
  e.initializeMesh();
  std::vector<float> init(334, 1e9f);
  init[5] = 0.f;
  EXPECT_NO_THROW(e.initializeVertices(init));
  EXPECT_NO_THROW(e.solveEikonal());
  if (fin(e).empty()) return;
  EXPECT(fin(e)[5] == 0.f);
  const float before = fin(e)[0];
  e.initSpeedMtxMultipliers(std::vector<float>(1125, 0.25f));  // metric 1/4: speed 2
  EXPECT_NO_THROW(e.solveEikonal());
  if (fin(e).empty()) return;
  EXPECT(std::fabs(fin(e)[0] - 0.5f * before) <= 1e-3f * before);
  EXPECT(e.stats().iterations > 0);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("usage: %s <fixture dir>\n", argv[0]);
    return 2;
  }
  std::setvbuf(stdout, nullptr, _IONBF, 0);
  D = std::string(argv[1]) + "/";
  small3d();
  basic3d();
  converge3d(false);
  converge3d(true);
  sanity3d();
  basic2d();
  sanity_converge2d();
  seeds_and_speeds();
  std::printf("%d checks, %d failed\n", g_checks, g_fail);
  return g_fail ? 1 : 0;
}
