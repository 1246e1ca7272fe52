// ref_harness.cpp -- C entry points into the reference's OWN source code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference sources that build without their third-party libraries:
//   include/xdg/geometry/plucker.h      (header; Plucker ray-triangle test)
//   src/geometry/closest.cpp            (closest point on a triangle)
//   src/mesh_manager_interface.cpp      (next_element / walk_elements)
//   src/config.cpp, src/error.cpp       (linked in by the above)
// into oracle/_ref/libxdg_ref.so.  The tests use it to pin the C restatement
// in oracle/xdg_oracle.c bit for bit and to write the golden fixtures under
// tests/golden/.  Nothing here is product code.
//
// HarnessMesh is a minimal in-memory MeshManager holding one tet mesh; only
// the methods the walk reads are meaningful.
#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <vector>

#include "xdg/constants.h"
#include "xdg/element_face_accessor.h"
#include "xdg/geometry/closest.h"
#include "xdg/geometry/plucker.h"
#include "xdg/mesh_manager_interface.h"
#include "xdg/vec3da.h"

using namespace xdg;

namespace {

class HarnessMesh : public MeshManager {
public:
  std::vector<Vertex> xyz;
  std::vector<std::array<int, 4>> conn;
  std::vector<std::array<int, 4>> adj;
  std::array<std::array<int, 3>, 4> faces;

  void load_file(const std::string&) override {}
  void init() override {}
  int num_volumes() const override { return 1; }
  int num_surfaces() const override { return 0; }
  int num_ents_of_dimension(int) const override { return 0; }
  int num_vertices() const override { return (int)xyz.size(); }
  int num_volume_elements(MeshID) const override { return (int)conn.size(); }
  int num_volume_faces(MeshID) const override { return 0; }
  int num_surface_faces(MeshID) const override { return 0; }
  std::vector<MeshID> get_volume_elements(MeshID) const override {
    std::vector<MeshID> v(conn.size());
    for (size_t i = 0; i < v.size(); ++i) v[i] = (MeshID)i;
    return v;
  }
  std::vector<MeshID> get_surface_faces(MeshID) const override { return {}; }
  std::vector<Vertex> element_vertices(MeshID e) const override {
    const auto& c = conn.at(e);
    return {xyz[c[0]], xyz[c[1]], xyz[c[2]], xyz[c[3]]};
  }
  std::array<Vertex, 3> face_vertices(MeshID) const override {
    throw std::runtime_error("no surface faces in the harness mesh");
  }
  SurfaceElementType get_surface_element_type(MeshID) const override {
    return SurfaceElementType::TRI;
  }
  MeshID adjacent_element(MeshID e, int face) const override { return adj.at(e).at(face); }
  double element_volume(MeshID) const override { return 0.0; }
  Vertex vertex_coordinates(MeshID v) const override { return xyz.at(v); }
  std::vector<MeshID> element_connectivity(MeshID e) const override {
    return {conn[e][0], conn[e][1], conn[e][2], conn[e][3]};
  }
  std::vector<MeshID> face_connectivity(MeshID) const override { return {}; }
  MeshID get_boundary_face_element(MeshID) const override { return ID_NONE; }
  std::vector<MeshID> get_volume_surfaces(MeshID) const override { return {}; }
  std::pair<MeshID, MeshID> surface_senses(MeshID) const override { return {ID_NONE, ID_NONE}; }
  Sense surface_sense(MeshID, MeshID) const override { return Sense::UNSET; }
  MeshID create_volume() override { return ID_NONE; }
  void add_surface_to_volume(MeshID, MeshID, Sense, bool) override {}
  void parse_metadata() override {}
  MeshLibrary mesh_library() const override { return MeshLibrary::MOCK; }
};

struct HarnessFaceAccessor : public ElementFaceAccessor {
  HarnessFaceAccessor(const HarnessMesh* m, MeshID e) : ElementFaceAccessor(e), mesh(m) {}
  std::array<Vertex, 3> face_vertices(int i) const override {
    const auto& c = mesh->conn.at(element_);
    const auto& f = mesh->faces[i];
    return {mesh->xyz[c[f[0]]], mesh->xyz[c[f[1]]], mesh->xyz[c[f[2]]]};
  }
  const HarnessMesh* mesh;
};

Vertex vtx(const double* p) { return Vertex(p[0], p[1], p[2]); }

} // namespace

// The reference defines this factory in element_face_accessor.cpp, which
// includes a test header that is not part of the tree; the harness supplies
// its own factory for its own mesh type.
std::shared_ptr<ElementFaceAccessor>
ElementFaceAccessor::create(const MeshManager* mm, MeshID element) {
  return std::make_shared<HarnessFaceAccessor>(dynamic_cast<const HarnessMesh*>(mm), element);
}

extern "C" {

double ref_plucker_edge_test(const double* va, const double* vb, const double* ray,
                             const double* rn) {
  return plucker_edge_test(vtx(va), vtx(vb), vtx(ray), vtx(rn));
}

int ref_plucker_ray_tri(const double* v, const double* o, const double* d, double tmax,
                        double tmin, int use_or, int orient, double* t_out) {
  dp::vec3 verts[3] = {vtx(v), vtx(v + 3), vtx(v + 6)};
  auto r = plucker_ray_tri_intersect(verts, vtx(o), vtx(d), tmax, tmin, use_or != 0, orient);
  if (r.hit && t_out) *t_out = r.t;
  return r.hit ? 1 : 0;
}

void ref_closest_on_tri(const double* v, const double* p, double* out) {
  std::array<Position, 3> tri {vtx(v), vtx(v + 3), vtx(v + 6)};
  Position r = closest_location_on_triangle(tri, vtx(p));
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

int ref_closest_region(const double* v, const double* p) {
  std::array<Position, 3> tri {vtx(v), vtx(v + 3), vtx(v + 6)};
  return static_cast<int>(determine_region(tri, vtx(p)));
}

void ref_normalize(double* v) {
  Vec3da a = vtx(v);
  a.normalize();
  v[0] = a.x; v[1] = a.y; v[2] = a.z;
}

void* ref_mesh_create(int64_t n_vert, const double* xyz, int64_t n_tet, const int32_t* conn,
                      const int32_t* adj, const int32_t* face_table) {
  auto* m = new HarnessMesh();
  m->xyz.resize(n_vert);
  for (int64_t i = 0; i < n_vert; ++i) m->xyz[i] = vtx(xyz + 3 * i);
  m->conn.resize(n_tet);
  m->adj.resize(n_tet);
  for (int64_t i = 0; i < n_tet; ++i)
    for (int k = 0; k < 4; ++k) {
      m->conn[i][k] = conn[4 * i + k];
      m->adj[i][k] = adj[4 * i + k];
    }
  for (int f = 0; f < 4; ++f)
    for (int k = 0; k < 3; ++k) m->faces[f][k] = face_table[3 * f + k];
  return m;
}

void ref_mesh_destroy(void* m) { delete static_cast<HarnessMesh*>(m); }

// MeshManager::next_element (mesh_manager_interface.cpp:149-200).  Callers
// must only pass cases where some face is exited (the reference indexes the
// adjacency with -1 otherwise).
int ref_next_element(void* m, int32_t elem, const double* r, const double* u, int32_t* next,
                     double* dist) {
  auto res = static_cast<HarnessMesh*>(m)->next_element(elem, vtx(r), vtx(u));
  *next = res.first;
  *dist = res.second;
  return 0;
}

// MeshManager::walk_elements (mesh_manager_interface.cpp:106-136)
int32_t ref_walk_elements(void* m, int32_t elem, const double* start, const double* u,
                          double distance, int32_t max_segs, int32_t* seg_elem,
                          double* seg_len) {
  auto segs = static_cast<HarnessMesh*>(m)->walk_elements(elem, vtx(start), vtx(u), distance);
  int32_t k = 0;
  for (const auto& s : segs) {
    if (k >= max_segs) break;
    seg_elem[k] = s.first;
    seg_len[k] = s.second;
    ++k;
  }
  return (int32_t)segs.size();
}

// MeshManager::walk_elements(start, end) overload (mesh_manager_interface.cpp:138-147)
int32_t ref_walk_elements_to(void* m, int32_t elem, const double* start, const double* end,
                             int32_t max_segs, int32_t* seg_elem, double* seg_len) {
  auto segs = static_cast<HarnessMesh*>(m)->walk_elements(elem, vtx(start), vtx(end));
  int32_t k = 0;
  for (const auto& s : segs) {
    if (k >= max_segs) break;
    seg_elem[k] = s.first;
    seg_len[k] = s.second;
    ++k;
  }
  return (int32_t)segs.size();
}

} // extern "C"
