// The reference's MeshMock Catch2 tests, replayed through the C++ backend
// class xdg::CudaRayTracer (the RayTracer subclass over the C ABI), in both
// precisions.  Exit status 0 when every check passes.
//
// Built two ways:
//  - against the stand-in declarations of xdg_api.h: the mesh below restates
//    the MeshMock fixture (tests/mesh_mock.h:17-321), a box
//    [-2,5]x[-3,6]x[-4,7] of six two-triangle surfaces, forward-sensed to
//    volume 0, split into twelve tets around the centre;
//  - with XDGCU_WITH_XDG_HEADERS, against XDG's own headers: the backend
//    derives from XDG's RayTracer and the tests run on the reference's own
//    MeshMock (include/xdg/testing/mesh_mock.h) and its ElementFaceAccessor
//    factory (src/element_face_accessor.cpp), linked from XDG's sources.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <thread>
#include <vector>

#include "cuda_ray_tracer.h"
#ifdef XDGCU_WITH_XDG_HEADERS
#include "xdg/testing/mesh_mock.h"
#endif

using namespace xdg;

namespace {

int g_failures = 0;
int g_checks = 0;

#define CHECK(cond)                                                            \
  do {                                                                         \
    ++g_checks;                                                                \
    if (!(cond)) {                                                             \
      ++g_failures;                                                            \
      std::fprintf(stderr, "%s:%d: CHECK failed: %s\n", __FILE__, __LINE__, #cond); \
    }                                                                          \
  } while (0)

#define CHECK_NEAR(a, b, tol) CHECK(std::fabs((a) - (b)) < (tol))

constexpr double LO[3] = {-2.0, -3.0, -4.0};
constexpr double HI[3] = {5.0, 6.0, 7.0};

// upper z plane, lower z plane, centre (mesh_mock.h:251-263)
const double VERTS[9][3] = {
    {HI[0], LO[1], HI[2]}, {HI[0], HI[1], HI[2]}, {LO[0], HI[1], HI[2]},
    {LO[0], LO[1], HI[2]}, {HI[0], LO[1], LO[2]}, {HI[0], HI[1], LO[2]},
    {LO[0], HI[1], LO[2]}, {LO[0], LO[1], LO[2]},
    {0.5 * (LO[0] + HI[0]), 0.5 * (LO[1] + HI[1]), 0.5 * (LO[2] + HI[2])}};

const int TRIS[12][3] = {{0, 1, 2}, {0, 2, 3}, {4, 6, 5}, {4, 7, 6}, {0, 5, 1}, {0, 4, 5},
                         {2, 6, 7}, {2, 7, 3}, {1, 5, 6}, {1, 6, 2}, {0, 7, 4}, {0, 3, 7}};

const int TETS[12][4] = {{0, 1, 2, 8}, {0, 2, 3, 8}, {4, 6, 5, 8}, {4, 7, 6, 8},
                         {0, 5, 1, 8}, {0, 4, 5, 8}, {2, 6, 7, 8}, {2, 7, 3, 8},
                         {0, 7, 4, 8}, {0, 3, 7, 8}, {1, 5, 6, 8}, {1, 6, 2, 8}};

const int ADJ[12][4] = {{-1, 1, 4, 11}, {-1, 9, 0, 7}, {-1, 5, 3, 10}, {-1, 2, 8, 6},
                        {-1, 0, 5, 10}, {-1, 4, 8, 2}, {-1, 7, 11, 3}, {-1, 1, 6, 9},
                        {-1, 5, 9, 3},  {-1, 8, 1, 7}, {-1, 11, 4, 2}, {-1, 0, 10, 6}};

// MeshMock's tet faces in its canonical order
const int TET_FACES[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};

Vertex vert(int i) { return {VERTS[i][0], VERTS[i][1], VERTS[i][2]}; }

#ifdef XDGCU_WITH_XDG_HEADERS

using MockMesh = ::MeshMock;  // the reference's own fixture

}  // namespace

#else

class MockMesh : public MeshManager {
 public:
  explicit MockMesh(bool volumetric) : volumetric_(volumetric) { volumes_ = {0}; }
  std::vector<MeshID> get_volume_surfaces(MeshID) const override { return {0, 1, 2, 3, 4, 5}; }
  std::vector<MeshID> get_surface_faces(MeshID s) const override { return {2 * s, 2 * s + 1}; }
  std::array<Vertex, 3> face_vertices(MeshID f) const override {
    return {vert(TRIS[f][0]), vert(TRIS[f][1]), vert(TRIS[f][2])};
  }
  std::pair<MeshID, MeshID> surface_senses(MeshID) const override { return {0, ID_NONE}; }
  // every volume holds all twelve tets (mesh_mock.h:77-80)
  std::vector<MeshID> get_volume_elements(MeshID) const override {
    if (!volumetric_) return {};
    std::vector<MeshID> e(12);
    for (int i = 0; i < 12; ++i) e[i] = i;
    return e;
  }
  std::vector<Vertex> element_vertices(MeshID e) const override {
    return {vert(TETS[e][0]), vert(TETS[e][1]), vert(TETS[e][2]), vert(TETS[e][3])};
  }
  std::vector<MeshID> element_connectivity(MeshID e) const override {
    return {TETS[e][0], TETS[e][1], TETS[e][2], TETS[e][3]};
  }
  Vertex vertex_coordinates(MeshID v) const override { return vert(v); }
  MeshID adjacent_element(MeshID e, int face) const override { return ADJ[e][face]; }
  MeshID get_boundary_face_element(MeshID) const override { return ID_NONE; }
  MeshLibrary mesh_library() const override { return MeshLibrary::MOCK; }

 private:
  bool volumetric_;
};

struct MockFaceAccessor : ElementFaceAccessor {
  MockFaceAccessor(const MeshManager* mm, MeshID e) : ElementFaceAccessor(e), mm_(mm) {}
  std::array<Vertex, 3> face_vertices(int i) const override {
    const std::vector<Vertex> v = mm_->element_vertices(element_);
    return {v[TET_FACES[i][0]], v[TET_FACES[i][1]], v[TET_FACES[i][2]]};
  }
  const MeshManager* mm_;
};

}  // namespace

// The mesh library's accessor factory (element_face_accessor.cpp); this
// program links only the mock library.
std::shared_ptr<ElementFaceAccessor> ElementFaceAccessor::create(const MeshManager* mm,
                                                                 MeshID element) {
  return std::make_shared<MockFaceAccessor>(mm, element);
}

#endif  // XDGCU_WITH_XDG_HEADERS

namespace {

// tests/test_ray_fire.cpp:19-111
void test_ray_fire(int prec) {
  auto mm = std::make_shared<MockMesh>(false);
  CudaRayTracer rti(0, prec);
  const auto trees = rti.register_volume(mm, 0);
  const TreeID vt = trees.first;
  CHECK(vt != TREE_NONE);
  CHECK(trees.second == TREE_NONE);
  const Position origin{0.0, 0.0, 0.0};
  const struct {
    Direction d;
    double t;
  } axes[] = {{{1, 0, 0}, 5.0}, {{-1, 0, 0}, 2.0}, {{0, 1, 0}, 6.0},
              {{0, -1, 0}, 3.0}, {{0, 0, 1}, 7.0}, {{0, 0, -1}, 4.0}};
  for (const auto& a : axes) CHECK_NEAR(rti.ray_fire(vt, origin, a.d).first, a.t, 1e-6);

  CHECK_NEAR(rti.ray_fire(vt, {-10, 0, 0}, {1, 0, 0}).first, 15.0, 1e-6);
  CHECK_NEAR(rti.ray_fire(vt, {10, 0, 0}, {-1, 0, 0}).first, 12.0, 1e-6);
  CHECK_NEAR(rti.ray_fire(vt, {-10, 0, 0}, {1, 0, 0}, INFTY, HitOrientation::ENTERING).first,
             8.0, 1e-6);
  CHECK_NEAR(rti.ray_fire(vt, {10, 0, 0}, {-1, 0, 0}, INFTY, HitOrientation::ENTERING).first,
             5.0, 1e-6);

  // distance limits
  CHECK(rti.ray_fire(vt, origin, {1, 0, 0}, 4.5).second == ID_NONE);
  auto hit = rti.ray_fire(vt, origin, {1, 0, 0}, 5.1);
  CHECK(hit.second != ID_NONE);
  CHECK_NEAR(hit.first, 5.0, 1e-6);

  // the hit face is appended to the exclusion list and then skipped
  std::vector<MeshID> exclude;
  hit = rti.ray_fire(vt, origin, {1, 0, 0}, INFTY, HitOrientation::EXITING, &exclude);
  CHECK_NEAR(hit.first, 5.0, 1e-6);
  CHECK(exclude.size() == 1);
  hit = rti.ray_fire(vt, origin, {1, 0, 0}, INFTY, HitOrientation::EXITING, &exclude);
  CHECK(hit.second == ID_NONE);
  CHECK(hit.first == INFTY);
  CHECK(exclude.size() == 1);
}

// tests/test_point_in_volume.cpp:17-79
void test_point_in_volume(int prec) {
  auto mm = std::make_shared<MockMesh>(false);
  CudaRayTracer rti(0, prec);
  const TreeID vt = rti.register_volume(mm, 0).first;
  CHECK(rti.point_in_volume(vt, {0, 0, 0}));
  CHECK(!rti.point_in_volume(vt, {0, 0, 1000}));
  CHECK(rti.point_in_volume(vt, {4.0 - 1e-6, 0, 0}));
  CHECK(!rti.point_in_volume(vt, {5.001, 0, 0}));
  const Direction px{1, 0, 0}, mx{-1, 0, 0};
  CHECK(rti.point_in_volume(vt, {5.0, 0, 0}, &px));
  CHECK(!rti.point_in_volume(vt, {5.1, 0, 0}, &px));
  CHECK(!rti.point_in_volume(vt, {5.1, 0, 0}, &mx));
  // an excluded primitive list is accepted
  std::vector<MeshID> exclude;
  CHECK(rti.point_in_volume(vt, {0, 0, 0}, nullptr, &exclude));
}

// tests/test_occluded.cpp:12-31
void test_occluded(int prec) {
  auto mm = std::make_shared<MockMesh>(true);
  CudaRayTracer rti(0, prec);
  const TreeID vt = rti.register_volume(mm, 0).first;
  double dist = 0.0;
  CHECK(rti.occluded(vt, {-100, 0, 0}, {1, 0, 0}, dist));
  CHECK(dist == -INFTY);
  CHECK(!rti.occluded(vt, {-100, 0, 0}, {-1, 0, 0}, dist));
  CHECK(dist == INFTY);
}

// tests/test_find_element.cpp:12-41 and the tree counts of tests/test_bvh.cpp:12-47
void test_find_element(int prec) {
  auto mm = std::make_shared<MockMesh>(true);
  CudaRayTracer rti(0, prec);
  const auto trees = rti.register_volume(mm, 0);
  CHECK(rti.num_registered_trees() == 2);
  CHECK(rti.num_registered_surface_trees() == 1);
  CHECK(rti.num_registered_element_trees() == 1);
  CHECK(rti.find_element(trees.second, {0, 0, 0}) != ID_NONE);
  CHECK(rti.find_element(trees.second, {10, 10, 10}) == ID_NONE);
  // every tet's centroid lies in that tet
  for (int e = 0; e < 12; ++e) {
    Position c;
    for (int k = 0; k < 4; ++k) c = c + vert(TETS[e][k]) * 0.25;
    CHECK(rti.find_element(trees.second, c) == e);
  }
  rti.create_global_surface_tree();
  rti.create_global_element_tree();
  CHECK(rti.num_registered_trees() == 4);
  CHECK(rti.find_element({0, 0, 0}) != ID_NONE);
  CHECK(rti.find_element({-10, 0, 0}) == ID_NONE);
}

// tests/test_closest.cpp:18-59 (the distances along the x axis)
void test_closest(int prec) {
  auto mm = std::make_shared<MockMesh>(true);
  CudaRayTracer rti(0, prec);
  const TreeID vt = rti.register_volume(mm, 0).first;
  CHECK_NEAR(rti.closest(vt, {0, 0, 0}).first, 2.0, 1e-6);
  CHECK_NEAR(rti.closest(vt, {4, 0, 0}).first, 1.0, 1e-6);
  CHECK_NEAR(rti.closest(vt, {10, 0, 0}).first, 5.0, 1e-6);
  const double cy = 0.5 * (LO[1] + HI[1]), cz = 0.5 * (LO[2] + HI[2]);
  for (int i = 0; i <= 40; ++i) {
    const double x = -10.0 + 0.5 * i;
    const double exp = x < 1.5 ? std::fabs(x - LO[0]) : std::fabs(x - HI[0]);
    CHECK_NEAR(rti.closest(vt, {x, cy, cz}).first, exp, 1e-6);
  }
}

// tests/test_tally_segments.cpp:15-72: next_element from (-1,-2,-3) to the
// upper corner, then the same track as one walk_elements call
void test_walk(int prec) {
  auto mm = std::make_shared<MockMesh>(true);
  CudaRayTracer rti(0, prec);
  rti.register_volume(mm, 0);
  rti.create_global_element_tree();
  Position r{-1.0, -2.0, -3.0};
  const Position corner{HI[0], HI[1], HI[2]};
  const Position w = corner - r;
  double distance = w.length();
  const Direction u = w * (1.0 / distance);
  const Position start = r;
  const double total = distance;
  MeshID elem = rti.find_element(r);
  const MeshID first = elem;
  CHECK(elem != ID_NONE);
  int iters = 0;
  double summed = 0.0;
  while (elem != ID_NONE && iters < 100) {
    const auto nx = rti.next_element(elem, r, u);
    CHECK(nx.second < distance + 1e-9);
    r = r + u * nx.second;
    distance -= nx.second;
    summed += nx.second;
    elem = nx.first;
    ++iters;
  }
  CHECK(iters < 100);
  CHECK(elem == ID_NONE);
  for (int k = 0; k < 3; ++k) CHECK(std::fabs(r[k] - corner[k]) <= 1e-4 * std::fabs(corner[k]));

  const auto segs = rti.walk_elements(first, start, u, total);
  CHECK(!segs.empty());
  double walked = 0.0;
  for (const auto& s : segs) {
    CHECK(s.first >= 0 && s.first < 12);
    CHECK(s.second >= 0.0);
    walked += s.second;
  }
  CHECK(std::fabs(walked - total) <= 1e-9 * total);
  CHECK(std::fabs(walked - summed) <= 1e-9 * total);
}

// The batched entry point over host arrays agrees with the scalar method.
void test_batch(int prec) {
  auto mm = std::make_shared<MockMesh>(false);
  CudaRayTracer rti(0, prec);
  const TreeID vt = rti.register_volume(mm, 0).first;
  const int n = 64;
  std::vector<double> org(3 * n), dir(3 * n), dl(n, INFTY), t(n);
  std::vector<int32_t> surf(n), face(n);
  for (int i = 0; i < n; ++i) {
    const double a = 0.1 * i, b = 0.37 * i;
    org[3 * i] = 0.01 * i;
    org[3 * i + 1] = -0.02 * i;
    org[3 * i + 2] = 0.03 * i;
    dir[3 * i] = std::cos(a) * std::sin(b);
    dir[3 * i + 1] = std::sin(a) * std::sin(b);
    dir[3 * i + 2] = std::cos(b);
  }
  rti.ray_fire_batch(vt, nullptr, n, org.data(), dir.data(), dl.data(), HitOrientation::EXITING,
                     t.data(), surf.data(), face.data());
  std::vector<int32_t> inside(n);
  rti.point_in_volume_batch(vt, nullptr, n, org.data(), nullptr, inside.data());
  for (int i = 0; i < n; ++i) {
    const Position o{org[3 * i], org[3 * i + 1], org[3 * i + 2]};
    const Direction d{dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
    const auto hit = rti.ray_fire(vt, o, d);
    CHECK(hit.first == t[i]);
    CHECK(hit.second == surf[i]);
    CHECK(surf[i] != ID_NONE);
    CHECK(inside[i] == (rti.point_in_volume(vt, o) ? 1 : 0));
  }
}

// The scalar methods called concurrently from several host threads on one
// backend object, as the reference's OpenMP loops call them
// (tools/ray_benchmark.cpp:209-213): every result equals the batched call's
// (ray_fire, point_in_volume) or the single-threaded scalar call's
// (find_element).
void test_threads(int prec) {
  auto mm = std::make_shared<MockMesh>(true);
  CudaRayTracer rti(0, prec);
  const auto trees = rti.register_volume(mm, 0);
  const TreeID vt = trees.first, et = trees.second;
  const int nth = 8, per = 300, n = nth * per;
  std::vector<double> org(3 * n), dir(3 * n), dl(n, INFTY), t(n);
  std::vector<int32_t> surf(n), face(n), inside(n);
  unsigned long long s = 12345;
  auto uni = [&s]() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) org[3 * i + c] = LO[c] + 0.05 + (HI[c] - LO[c] - 0.1) * uni();
    double d[3], len = 0.0;
    do {
      len = 0.0;
      for (int c = 0; c < 3; ++c) {
        d[c] = 2.0 * uni() - 1.0;
        len += d[c] * d[c];
      }
    } while (len > 1.0 || len < 1e-6);
    len = std::sqrt(len);
    for (int c = 0; c < 3; ++c) dir[3 * i + c] = d[c] / len;
  }
  rti.ray_fire_batch(vt, nullptr, n, org.data(), dir.data(), dl.data(), HitOrientation::EXITING,
                     t.data(), surf.data(), face.data());
  rti.point_in_volume_batch(vt, nullptr, n, org.data(), nullptr, inside.data());
  std::vector<double> tt(n);
  std::vector<MeshID> ss(n), ee(n);
  std::vector<int> in(n);
  std::vector<std::thread> pool;
  for (int k = 0; k < nth; ++k)
    pool.emplace_back([&, k] {
      for (int i = k * per; i < (k + 1) * per; ++i) {
        const Position o{org[3 * i], org[3 * i + 1], org[3 * i + 2]};
        const Direction d{dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
        const auto h = rti.ray_fire(vt, o, d);
        tt[i] = h.first;
        ss[i] = h.second;
        in[i] = rti.point_in_volume(vt, o) ? 1 : 0;
        ee[i] = rti.find_element(et, o);
      }
    });
  for (auto& th : pool) th.join();
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    const Position o{org[3 * i], org[3 * i + 1], org[3 * i + 2]};
    if (tt[i] != t[i] || ss[i] != surf[i] || in[i] != inside[i] || ee[i] != rti.find_element(et, o))
      ++bad;
    if (ss[i] == ID_NONE || in[i] != 1 || ee[i] == ID_NONE) ++bad;
  }
  CHECK(bad == 0);
}

}  // namespace

int main() {
  for (int prec : {XDGCU_FP64, XDGCU_MIXED}) {
    test_ray_fire(prec);
    test_point_in_volume(prec);
    test_occluded(prec);
    test_find_element(prec);
    test_closest(prec);
    test_walk(prec);
    test_batch(prec);
    test_threads(prec);
  }
  std::printf("%d checks, %d failures\n", g_checks, g_failures);
  return g_failures == 0 ? 0 : 1;
}
