// cuda_ray_tracer.cpp -- XDG RayTracer backend over the C ABI of the GB300
// engine.  Geometry is read through MeshManager exactly where
// EmbreeRayTracer reads it (embree/ray_tracer.cpp:38-188); queries forward to
// the batched C entry points, with n = 1 for the scalar RayTracer methods.
#include "cuda_ray_tracer.h"

#include <cstdio>
#include <stdexcept>

namespace xdg {

namespace {

void to3(const Vec3da& v, double* out) {
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
}

}  // namespace

CudaRayTracer::CudaRayTracer(int device, int precision) : precision_(precision) {
  check(xdgcu_create(&ctx_, device), "xdgcu_create");
}

CudaRayTracer::~CudaRayTracer() {
  if (ctx_) xdgcu_destroy(ctx_);
}

void CudaRayTracer::check(int rc, const char* what) const {
  if (rc != XDGCU_OK)
    throw std::runtime_error(std::string(what) + ": " + xdgcu_last_error(ctx_));
}

std::pair<TreeID, TreeID> CudaRayTracer::register_volume(const std::shared_ptr<MeshManager>& mm,
                                                         MeshID volume) {
  // embree/ray_tracer.cpp:38-47
  const TreeID faces_tree = create_surface_tree(mm, volume);
  const TreeID element_tree = create_element_tree(mm, volume);
  return {faces_tree, element_tree};
}

TreeID CudaRayTracer::create_surface_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) {
  // embree/ray_tracer.cpp:49-105: first visit registers the surface's faces,
  // every visit records which sense the volume has on it
  const std::vector<MeshID> surfaces = mm->get_volume_surfaces(volume);
  std::vector<int32_t> ids, sense;
  for (MeshID s : surfaces) {
    if (!registered_surfaces_.count(s)) {
      const std::vector<MeshID> faces = mm->get_surface_faces(s);
      std::vector<double> xyz(9 * faces.size());
      std::vector<int32_t> fid(faces.begin(), faces.end());
      for (size_t k = 0; k < faces.size(); ++k) {
        const std::array<Vertex, 3> v = mm->face_vertices(faces[k]);
        for (int j = 0; j < 3; ++j) to3(v[j], &xyz[9 * k + 3 * j]);
      }
      check(xdgcu_register_surface(ctx_, s, (int64_t)faces.size(), xyz.data(), fid.data()),
            "register_surface");
      registered_surfaces_.insert(s);
    }
    const std::pair<MeshID, MeshID> senses = mm->surface_senses(s);
    if (volume == senses.first) {
      sense.push_back(0);
    } else if (volume == senses.second) {
      sense.push_back(1);
    } else {
      throw std::runtime_error("Volume " + std::to_string(volume) + " is not a parent of surface " +
                               std::to_string(s));
    }
    ids.push_back(s);
  }
  TreeID tree = TREE_NONE;
  check(xdgcu_create_surface_tree(ctx_, ids.data(), sense.data(), (int32_t)ids.size(),
                                  bounding_box_bump(mm, volume), &tree),
        "create_surface_tree");
  claim_surface_tree_id(tree);
  surface_trees_.push_back(tree);
  return tree;
}

void CudaRayTracer::upload_tet_mesh(const MeshManager* mm) {
  // every element of every volume, in volume order
  std::vector<MeshID> elems;
  for (MeshID v : mm->volumes())
    for (MeshID e : mm->get_volume_elements(v))
      if (!tet_index_.count(e)) {
        tet_index_[e] = (int32_t)elems.size();
        elems.push_back(e);
      }
  tet_ids_ = elems;
  std::unordered_map<MeshID, int32_t> vidx;
  std::vector<double> xyz;
  std::vector<int32_t> conn(4 * elems.size()), adj(4 * elems.size());
  for (size_t k = 0; k < elems.size(); ++k) {
    const std::vector<MeshID> c = mm->element_connectivity(elems[k]);
    if (c.size() != 4) throw std::runtime_error("CUDA backend: only tetrahedra are supported");
    for (int j = 0; j < 4; ++j) {
      auto it = vidx.find(c[j]);
      if (it == vidx.end()) {
        it = vidx.emplace(c[j], (int32_t)(xyz.size() / 3)).first;
        const Vertex p = mm->vertex_coordinates(c[j]);
        xyz.push_back(p.x);
        xyz.push_back(p.y);
        xyz.push_back(p.z);
      }
      conn[4 * k + j] = it->second;
      const MeshID nb = mm->adjacent_element(elems[k], j);
      auto nt = tet_index_.find(nb);
      adj[4 * k + j] = (nb == ID_NONE || nt == tet_index_.end()) ? -1 : nt->second;
    }
  }
  // local face table of the library's ElementFaceAccessor, by matching the
  // face vertices against the element's vertices
  int32_t faces[12] = {0, 1, 3, 1, 2, 3, 2, 0, 3, 0, 2, 1};
  if (!elems.empty()) {
    const std::vector<Vertex> ev = mm->element_vertices(elems[0]);
    const std::shared_ptr<ElementFaceAccessor> acc = ElementFaceAccessor::create(mm, elems[0]);
    for (int f = 0; f < 4; ++f) {
      const std::array<Vertex, 3> fv = acc->face_vertices(f);
      for (int j = 0; j < 3; ++j) {
        int found = -1;
        for (int k = 0; k < 4; ++k)
          if (fv[j].x == ev[k].x && fv[j].y == ev[k].y && fv[j].z == ev[k].z) found = k;
        if (found < 0) throw std::runtime_error("CUDA backend: cannot derive the tet face order");
        faces[3 * f + j] = found;
      }
    }
  }
  std::vector<int32_t> ids(elems.begin(), elems.end());
  check(xdgcu_set_tet_mesh(ctx_, (int64_t)(xyz.size() / 3), xyz.data(), (int64_t)elems.size(),
                           conn.data(), adj.data(), ids.data(), faces),
        "set_tet_mesh");
  tets_uploaded_ = true;
}

TreeID CudaRayTracer::create_element_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) {
  // embree/ray_tracer.cpp:149-188
  const std::vector<MeshID> elements = mm->get_volume_elements(volume);
  if (elements.empty()) return TREE_NONE;
  if (!tets_uploaded_) upload_tet_mesh(mm.get());
  std::vector<int32_t> idx;
  idx.reserve(elements.size());
  for (MeshID e : elements) idx.push_back(tet_index(e));
  TreeID tree = TREE_NONE;
  check(xdgcu_create_element_tree(ctx_, idx.data(), (int64_t)idx.size(), &tree),
        "create_element_tree");
  claim_element_tree_id(tree);
  element_trees_.push_back(tree);
  return tree;
}

void CudaRayTracer::create_global_surface_tree() {
  TreeID tree = TREE_NONE;
  check(xdgcu_create_global_surface_tree(ctx_, &tree), "create_global_surface_tree");
  claim_surface_tree_id(tree);
  surface_trees_.push_back(tree);
  global_surface_tree_ = tree;
}

void CudaRayTracer::create_global_element_tree() {
  TreeID tree = TREE_NONE;
  check(xdgcu_create_global_element_tree(ctx_, &tree), "create_global_element_tree");
  claim_element_tree_id(tree);
  element_trees_.push_back(tree);
  global_element_tree_ = tree;
}

// The engine numbers each kind of tree from 1 in creation order, as the base
// class's counters do (ray_tracing_interface.cpp:10-18); the backend takes
// the base class's next id and checks that the engine gave the same one.
void CudaRayTracer::claim_surface_tree_id(TreeID tree) {
  if (tree != next_surface_tree_id())
    throw std::runtime_error("CUDA backend: surface tree ids out of step with the engine");
}

void CudaRayTracer::claim_element_tree_id(TreeID tree) {
  if (tree != next_element_tree_id())
    throw std::runtime_error("CUDA backend: element tree ids out of step with the engine");
}

int32_t CudaRayTracer::tet_index(MeshID element) const {
  auto it = tet_index_.find(element);
  if (it == tet_index_.end())
    throw std::runtime_error("element " + std::to_string(element) + " is not in any element tree");
  return it->second;
}

bool CudaRayTracer::point_in_volume(TreeID tree, const Position& point, const Direction* direction,
                                    const std::vector<MeshID>* exclude) const {
  double p[3], d[3];
  to3(point, p);
  if (direction) to3(*direction, d);
  int32_t off[2] = {0, exclude ? (int32_t)exclude->size() : 0};
  int32_t dummy = 0;
  const int32_t* ids = exclude && !exclude->empty() ? exclude->data() : &dummy;
  int32_t inside = 0;
  check(xdgcu_point_in_volume(ctx_, tree, nullptr, 1, p, direction ? d : nullptr,
                              exclude ? off : nullptr, exclude ? ids : nullptr, &inside, nullptr,
                              precision_, nullptr),
        "point_in_volume");
  return inside != 0;
}

std::pair<double, MeshID> CudaRayTracer::ray_fire(TreeID tree, const Position& origin,
                                                  const Direction& direction,
                                                  const double dist_limit,
                                                  HitOrientation orientation,
                                                  std::vector<MeshID>* const exclude) {
  double o[3], d[3], dl = dist_limit, t = INFTY;
  to3(origin, o);
  to3(direction, d);
  int32_t off[2] = {0, exclude ? (int32_t)exclude->size() : 0};
  int32_t dummy = 0;
  const int32_t* ids = exclude && !exclude->empty() ? exclude->data() : &dummy;
  int32_t surf = ID_NONE, face = ID_NONE;
  check(xdgcu_ray_fire(ctx_, tree, nullptr, 1, o, d, &dl, (int32_t)orientation,
                       exclude ? off : nullptr, exclude ? ids : nullptr, &t, &surf, &face, nullptr,
                       precision_, nullptr),
        "ray_fire");
  if (surf == ID_NONE) return {INFTY, ID_NONE};
  if (exclude) exclude->push_back(face);  // embree/ray_tracer.cpp:324
  return {t, surf};
}

MeshID CudaRayTracer::find_element(const Position& point) const {
  return find_element(global_element_tree_, point);
}

MeshID CudaRayTracer::find_element(TreeID tree, const Position& point) const {
  if (tree < 1 || tree > xdgcu_num_element_trees(ctx_)) {
    // embree/ray_tracer.cpp:236-239
    std::fprintf(stderr, "Warning: Tree %d does not have a point location tree\n", tree);
    return ID_NONE;
  }
  double p[3];
  to3(point, p);
  int32_t id = ID_NONE;
  check(xdgcu_find_element(ctx_, tree, nullptr, 1, p, &id, nullptr, nullptr, precision_, nullptr),
        "find_element");
  return id;
}

std::pair<double, MeshID> CudaRayTracer::closest(TreeID tree, const Position& origin) {
  double p[3], dist = INFTY;
  to3(origin, p);
  int32_t face = ID_NONE;
  check(xdgcu_closest(ctx_, tree, nullptr, 1, p, &dist, &face, nullptr, precision_, nullptr),
        "closest");
  if (face == ID_NONE) return {INFTY, ID_NONE};
  return {dist, face};
}

bool CudaRayTracer::occluded(TreeID tree, const Position& origin, const Direction& direction,
                             double& dist) const {
  double o[3], d[3];
  to3(origin, o);
  to3(direction, d);
  int32_t occ = 0;
  check(xdgcu_occluded(ctx_, tree, nullptr, 1, o, d, &occ, &dist, nullptr, precision_, nullptr),
        "occluded");
  return occ != 0;
}

std::pair<MeshID, double> CudaRayTracer::next_element(MeshID element, const Position& r,
                                                      const Direction& u) const {
  const int32_t e = tet_index(element);
  double rr[3], uu[3], dist = INFTY;
  to3(r, rr);
  to3(u, uu);
  int32_t next = -1, st = 0;
  check(xdgcu_next_element(ctx_, 1, &e, rr, uu, &next, &dist, &st, precision_, nullptr),
        "next_element");
  return {next < 0 ? ID_NONE : tet_ids_[next], dist};
}

std::vector<std::pair<MeshID, double>> CudaRayTracer::walk_elements(MeshID element,
                                                                    const Position& start,
                                                                    const Direction& u,
                                                                    double distance) const {
  const int32_t e = tet_index(element);
  double s[3], uu[3];
  to3(start, s);
  to3(u, uu);
  int64_t offsets[2] = {0, 0};
  int32_t st = 0;
  // first call sizes the output, second fills it
  check(xdgcu_walk_elements_packed(ctx_, 1, &e, s, uu, &distance, 1 << 20, 0, nullptr, nullptr,
                                   offsets, &st, precision_, nullptr),
        "walk_elements");
  const int64_t total = offsets[1];
  std::vector<int32_t> elem(total > 0 ? total : 1);
  std::vector<double> len(total > 0 ? total : 1);
  check(xdgcu_walk_elements_packed(ctx_, 1, &e, s, uu, &distance, 1 << 20, total, elem.data(),
                                   len.data(), offsets, &st, precision_, nullptr),
        "walk_elements");
  std::vector<std::pair<MeshID, double>> out;
  out.reserve(total);
  for (int64_t k = 0; k < total; ++k) out.push_back({elem[k], len[k]});
  return out;
}

void CudaRayTracer::ray_fire_batch(TreeID tree, const int32_t* ray_trees, int64_t n,
                                   const double* origins, const double* directions,
                                   const double* dist_limits, HitOrientation orientation,
                                   double* t_out, int32_t* surface_out, int32_t* face_out,
                                   void* stream) const {
  check(xdgcu_ray_fire(ctx_, tree, ray_trees, n, origins, directions, dist_limits,
                       (int32_t)orientation, nullptr, nullptr, t_out, surface_out, face_out,
                       nullptr, precision_, stream),
        "ray_fire");
}

void CudaRayTracer::point_in_volume_batch(TreeID tree, const int32_t* ray_trees, int64_t n,
                                          const double* points, const double* directions,
                                          int32_t* inside_out, void* stream) const {
  check(xdgcu_point_in_volume(ctx_, tree, ray_trees, n, points, directions, nullptr, nullptr,
                              inside_out, nullptr, precision_, stream),
        "point_in_volume");
}

}  // namespace xdg
