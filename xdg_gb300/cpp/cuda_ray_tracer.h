// cuda_ray_tracer.h -- XDG RayTracer backend on the GB300 engine (C ABI in
// include/xdgcu.h).  Drop-in beside EmbreeRayTracer / GPRTRayTracer.
#pragma once

#include <mutex>
#include <set>
#include <string>
#include <unordered_map>

#include "xdg_api.h"
#include "xdgcu.h"

namespace xdg {

class CudaRayTracer : public RayTracer {
 public:
  // precision: XDGCU_MIXED (default; FP32 traversal with certified FP64
  // escalation) or XDGCU_FP64.  Both give bit-identical results.
  explicit CudaRayTracer(int device = 0, int precision = XDGCU_MIXED);
  ~CudaRayTracer() override;
  CudaRayTracer(const CudaRayTracer&) = delete;
  CudaRayTracer& operator=(const CudaRayTracer&) = delete;

  void init() override {}
  std::pair<TreeID, TreeID> register_volume(const std::shared_ptr<MeshManager>& mm,
                                            MeshID volume) override;
  TreeID create_surface_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) override;
  TreeID create_element_tree(const std::shared_ptr<MeshManager>& mm, MeshID volume) override;
  void create_global_surface_tree() override;
  void create_global_element_tree() override;

  bool point_in_volume(TreeID tree, const Position& point, const Direction* direction = nullptr,
                       const std::vector<MeshID>* exclude_primitives = nullptr) const override;
  std::pair<double, MeshID> ray_fire(TreeID tree, const Position& origin,
                                     const Direction& direction, const double dist_limit = INFTY,
                                     HitOrientation orientation = HitOrientation::EXITING,
                                     std::vector<MeshID>* const exclude_primitives = nullptr) override;
  MeshID find_element(const Position& point) const override;
  MeshID find_element(TreeID tree, const Position& point) const override;
  std::pair<double, MeshID> closest(TreeID tree, const Position& origin) override;
  bool occluded(TreeID tree, const Position& origin, const Direction& direction,
                double& dist) const override;
  RTLibrary library() const override { return XDGCU_RTLIBRARY; }

  // the global trees (TREE_NONE until created)
  SurfaceTreeID global_surface_tree_id() const { return global_surface_tree_; }
  ElementTreeID global_element_tree_id() const { return global_element_tree_; }

  // MeshManager::next_element / walk_elements on the device, for the mesh
  // of the element trees (mesh_manager_interface.cpp:106-200).
  std::pair<MeshID, double> next_element(MeshID element, const Position& r,
                                         const Direction& u) const;
  std::vector<std::pair<MeshID, double>> walk_elements(MeshID element, const Position& start,
                                                       const Direction& u, double distance) const;

  // Batched forms (host or device arrays of n rays; see xdgcu.h).
  void ray_fire_batch(TreeID tree, const int32_t* ray_trees, int64_t n, const double* origins,
                      const double* directions, const double* dist_limits,
                      HitOrientation orientation, double* t_out, int32_t* surface_out,
                      int32_t* face_out, void* stream = nullptr) const;
  void point_in_volume_batch(TreeID tree, const int32_t* ray_trees, int64_t n,
                             const double* points, const double* directions, int32_t* inside_out,
                             void* stream = nullptr) const;

  xdgcu_ctx* context() const { return ctx_; }
  int precision() const { return precision_; }
  // the engine's tet index of an element of the element trees, and back
  int32_t tet_index(MeshID element) const;
  MeshID tet_id(int32_t index) const { return index < 0 ? ID_NONE : tet_ids_.at(index); }
  void check(int rc, const char* what) const;

 private:
  void upload_tet_mesh(const MeshManager* mm);
  void claim_surface_tree_id(TreeID tree);
  void claim_element_tree_id(TreeID tree);

  xdgcu_ctx* ctx_ = nullptr;
  int precision_;
  std::set<MeshID> registered_surfaces_;
  bool tets_uploaded_ = false;
  std::unordered_map<MeshID, int32_t> tet_index_;
  std::vector<MeshID> tet_ids_;
};

}  // namespace xdg
