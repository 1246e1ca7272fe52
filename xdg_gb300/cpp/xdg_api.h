// xdg_api.h -- XDG's public C++ interface as the CUDA backend sees it.
//
// Built with XDGCU_WITH_XDG_HEADERS defined (inside XDG, or against its
// source tree) this includes XDG's own headers:
//   xdg/constants.h, xdg/ray_tracing_interface.h, xdg/mesh_manager_interface.h,
//   xdg/element_face_accessor.h.
// Otherwise it declares the subset of them the backend uses, with the same
// names, signatures and protected state, so that the backend and its tests
// compile without the XDG tree.
//
// XDGCU_RTLIBRARY is the RTLibrary value the backend reports; XDG's
// integration adds CUDA to RTLibrary in constants.h, after EMBREE and GPRT.
#pragma once

#ifdef XDGCU_WITH_XDG_HEADERS

#include "xdg/constants.h"
#include "xdg/element_face_accessor.h"
#include "xdg/mesh_manager_interface.h"
#include "xdg/ray_tracing_interface.h"

#ifndef XDGCU_RTLIBRARY
#define XDGCU_RTLIBRARY ::xdg::RTLibrary::CUDA
#endif

#else  // the stand-in declarations

#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#ifndef XDGCU_RTLIBRARY
#define XDGCU_RTLIBRARY ::xdg::RTLibrary::CUDA
#endif

namespace xdg {

// constants.h:15, 73-87
constexpr double INFTY{DBL_MAX};
using MeshID = int32_t;
using TreeID = int32_t;
using SurfaceTreeID = TreeID;
using ElementTreeID = TreeID;
constexpr MeshID ID_NONE{-1};
constexpr TreeID TREE_NONE{-1};
constexpr double TINY_BIT{1e-10};  // constants.h:32

// shared_enums.h:11-15
enum HitOrientation : int { ANY = -1, EXITING = 0, ENTERING = 1 };
enum class Sense { UNSET = -1, FORWARD = 0, REVERSE = 1 };
enum class MeshLibrary { MOCK = 0, MOAB, LIBMESH };
enum class RTLibrary { EMBREE, GPRT, CUDA };  // CUDA: the integration adds it

// The subset of Vec3da (vec3da.h) the backend uses.
struct Vec3da {
  double x = 0.0, y = 0.0, z = 0.0;
  Vec3da() = default;
  Vec3da(double a, double b, double c) : x(a), y(b), z(c) {}
  double operator[](size_t i) const { return i == 0 ? x : (i == 1 ? y : z); }
  double& operator[](size_t i) { return i == 0 ? x : (i == 1 ? y : z); }
  double dot(const Vec3da& o) const { return x * o.x + y * o.y + z * o.z; }
  double length() const { return std::sqrt(x * x + y * y + z * z); }
};
inline Vec3da operator-(const Vec3da& a, const Vec3da& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3da operator+(const Vec3da& a, const Vec3da& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3da operator*(const Vec3da& a, double s) { return {s * a.x, s * a.y, s * a.z}; }
inline Vec3da operator*(double s, const Vec3da& a) { return {s * a.x, s * a.y, s * a.z}; }
inline Vec3da operator-(const Vec3da& a) { return {-a.x, -a.y, -a.z}; }
using Position = Vec3da;
using Direction = Vec3da;
using Vertex = Vec3da;

// bbox.h: BoundingBox with dilation() = max_chord_length() * FP_BOX_TOL
struct BoundingBox {
  double min_x = 0.0, min_y = 0.0, min_z = 0.0, max_x = 0.0, max_y = 0.0, max_z = 0.0;
  void update(const Vertex& v) {
    min_x = std::min(min_x, v.x);
    min_y = std::min(min_y, v.y);
    min_z = std::min(min_z, v.z);
    max_x = std::max(max_x, v.x);
    max_y = std::max(max_y, v.y);
    max_z = std::max(max_z, v.z);
  }
  double max_chord_length() const {
    const double wx = max_x - min_x, wy = max_y - min_y, wz = max_z - min_z;
    return std::sqrt(wx * wx + wy * wy + wz * wz);
  }
  double dilation() const { return max_chord_length() * 1e-6; }
};

// constants.h:95-113
enum class PropertyType { BOUNDARY_CONDITION = -1, MATERIAL = 0, DENSITY = 1, TEMPERATURE = 2 };
struct Property {
  PropertyType type;
  std::string value;
};

// The MeshManager queries a ray tracer and the tools read
// (mesh_manager_interface.h).
class MeshManager {
 public:
  virtual ~MeshManager() = default;
  virtual std::vector<MeshID> get_volume_surfaces(MeshID volume) const = 0;
  virtual std::vector<MeshID> get_surface_faces(MeshID surface) const = 0;
  virtual std::array<Vertex, 3> face_vertices(MeshID face) const = 0;
  virtual std::pair<MeshID, MeshID> surface_senses(MeshID surface) const = 0;
  virtual std::vector<MeshID> get_volume_elements(MeshID volume) const = 0;
  virtual std::vector<Vertex> element_vertices(MeshID element) const = 0;
  virtual std::vector<MeshID> element_connectivity(MeshID element) const = 0;
  virtual Vertex vertex_coordinates(MeshID vertex) const = 0;
  virtual MeshID adjacent_element(MeshID element, int face) const = 0;
  // the element owning a boundary face, ID_NONE if none
  // (mesh_manager_interface.h:153-157)
  virtual MeshID get_boundary_face_element(MeshID face) const = 0;
  virtual MeshLibrary mesh_library() const = 0;
  const std::vector<MeshID>& volumes() const { return volumes_; }
  const std::vector<MeshID>& surfaces() const { return surfaces_; }
  MeshID implicit_complement() const { return implicit_complement_; }
  // mesh_manager_interface.cpp: the forward-sense parent, then the reverse
  std::pair<MeshID, MeshID> get_parent_volumes(MeshID surface) const {
    return surface_senses(surface);
  }
  // mesh_manager_interface.cpp:98-104
  Property get_surface_property(MeshID surface, PropertyType type) const {
    auto it = surface_metadata_.find({surface, type});
    if (it == surface_metadata_.end()) return {PropertyType::BOUNDARY_CONDITION, "transmission"};
    return it->second;
  }
  // mesh_manager_interface.cpp:236-245: the box starts at zero
  BoundingBox volume_bounding_box(MeshID volume) const {
    BoundingBox bb;
    for (MeshID s : get_volume_surfaces(volume))
      for (MeshID f : get_surface_faces(s))
        for (const Vertex& v : face_vertices(f)) bb.update(v);
    return bb;
  }

 protected:
  std::vector<MeshID> volumes_;
  std::vector<MeshID> surfaces_;
  MeshID implicit_complement_{ID_NONE};
  std::map<std::pair<MeshID, PropertyType>, Property> surface_metadata_;
};

// element_face_accessor.h: face vertices of an element in the library's
// canonical face order.
struct ElementFaceAccessor {
  explicit ElementFaceAccessor(MeshID element) : element_(element) {}
  virtual ~ElementFaceAccessor() = default;
  static std::shared_ptr<ElementFaceAccessor> create(const MeshManager* mm, MeshID element);
  virtual std::array<Vertex, 3> face_vertices(int i) const = 0;
  MeshID element_;
};

// ray_tracing_interface.h:16-147
class RayTracer {
 public:
  virtual ~RayTracer() = default;
  virtual void init() = 0;
  virtual std::pair<TreeID, TreeID> register_volume(const std::shared_ptr<MeshManager>& mm,
                                                    MeshID volume) = 0;
  virtual TreeID create_surface_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) = 0;
  virtual TreeID create_element_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) = 0;
  virtual void create_global_surface_tree() = 0;
  virtual void create_global_element_tree() = 0;
  virtual bool point_in_volume(TreeID tree, const Position& point,
                               const Direction* direction = nullptr,
                               const std::vector<MeshID>* exclude_primitives = nullptr) const = 0;
  virtual std::pair<double, MeshID> ray_fire(TreeID tree, const Position& origin,
                                             const Direction& direction,
                                             const double dist_limit = INFTY,
                                             HitOrientation orientation = HitOrientation::EXITING,
                                             std::vector<MeshID>* const exclude_primitives = nullptr) = 0;
  virtual MeshID find_element(const Position& point) const = 0;
  virtual MeshID find_element(TreeID tree, const Position& point) const = 0;
  virtual std::pair<double, MeshID> closest(TreeID tree, const Position& origin) = 0;
  virtual bool occluded(TreeID tree, const Position& origin, const Direction& direction,
                        double& dist) const = 0;
  virtual RTLibrary library() const = 0;

  int num_registered_trees() const { return (int)(surface_trees_.size() + element_trees_.size()); }
  int num_registered_surface_trees() const { return (int)surface_trees_.size(); }
  int num_registered_element_trees() const { return (int)element_trees_.size(); }

 protected:
  // ray_tracing_interface.cpp:20-24
  double bounding_box_bump(const std::shared_ptr<MeshManager> mm, MeshID volume) {
    return std::max(mm->volume_bounding_box(volume).dilation(), numerical_precision_);
  }
  // ray_tracing_interface.cpp:10-18
  SurfaceTreeID next_surface_tree_id() { return ++next_surface_tree_id_; }
  ElementTreeID next_element_tree_id() { return ++next_element_tree_id_; }
  SurfaceTreeID global_surface_tree_{TREE_NONE};
  ElementTreeID global_element_tree_{TREE_NONE};
  std::map<MeshID, SurfaceTreeID> surface_to_tree_map_;
  std::map<MeshID, ElementTreeID> point_location_tree_map_;
  std::vector<SurfaceTreeID> surface_trees_;
  std::vector<ElementTreeID> element_trees_;
  SurfaceTreeID next_surface_tree_id_{0};
  ElementTreeID next_element_tree_id_{0};
  double numerical_precision_{1e-3};
};

}  // namespace xdg

#endif  // XDGCU_WITH_XDG_HEADERS
