// cuda_tools.cpp -- see cuda_tools.h.  All arrays are host arrays: the C ABI
// stages them through its per-thread device workspace.
#include "cuda_tools.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <stdexcept>

namespace xdg {

namespace {

// Vec3da::normalize (vec3da.h:61-66)
Vec3da normalized(Vec3da v) {
  double len = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  const double min_rcp = (double)(float)((double)FLT_MIN * 1e5);
  len = len < min_rcp ? min_rcp : len;
  return {v.x / len, v.y / len, v.z / len};
}

}  // namespace

void ParticleBank::resize(size_t n) {
  cell.resize(n, ID_NONE);
  pos.resize(3 * n);
  dir.resize(3 * n);
  rng.resize(n);
  distance.resize(n);
  events.resize(n);
  status.resize(n);
}

std::vector<uint64_t> seed_streams(uint64_t seed, size_t n) {
  std::vector<uint64_t> s(n);
  if (xdgcu_seed_streams(seed, (int64_t)n, s.data()) != XDGCU_OK)
    throw std::runtime_error(xdgcu_last_error(nullptr));
  return s;
}

// ---------------------------------------------------------------------------
// walk_elements tool
// ---------------------------------------------------------------------------

void walk_particles(CudaRayTracer& rt, TreeID ipc_surface_tree, ParticleBank& bank, double mfp,
                    int32_t max_events, std::vector<double>* element_tally, int max_reentries) {
  xdgcu_ctx* ctx = rt.context();
  const int prec = rt.precision();
  const size_t n = bank.size();
  std::vector<int32_t> idx(n);
  std::vector<char> ended(n);
  for (size_t i = 0; i < n; ++i) {
    idx[i] = bank.cell[i] == ID_NONE ? -1 : rt.tet_index(bank.cell[i]);
    ended[i] = idx[i] < 0;
  }
  double* tally = nullptr;
  if (element_tally) tally = element_tally->data();
  const TreeID gtree = rt.global_element_tree_id();
  for (int round = 0; round <= max_reentries; ++round) {
    rt.check(xdgcu_transport_elements(ctx, (int64_t)n, idx.data(), bank.pos.data(),
                                      bank.dir.data(), bank.rng.data(), mfp, max_events,
                                      bank.distance.data(), bank.events.data(), tally,
                                      bank.status.data(), prec, nullptr),
             "transport_elements");
    // particles that left the mesh in this launch look for re-entry
    // (walk_elements.h:88-94)
    std::vector<size_t> out;
    for (size_t i = 0; i < n; ++i)
      if (idx[i] < 0 && bank.status[i] == XDGCU_RAY_OK && !ended[i]) out.push_back(i);
    if (out.empty()) break;
    std::vector<std::vector<int32_t>> excl(out.size());
    std::vector<int32_t> found(out.size(), -1);
    std::vector<size_t> pend(out.size());
    for (size_t k = 0; k < out.size(); ++k) pend[k] = k;
    while (!pend.empty()) {
      const size_t m = pend.size();
      std::vector<double> o(3 * m), d(3 * m), t(m);
      std::vector<int32_t> off(m + 1, 0), ids, surf(m), face(m);
      for (size_t j = 0; j < m; ++j) {
        const size_t i = out[pend[j]];
        for (int c = 0; c < 3; ++c) {
          o[3 * j + c] = bank.pos[3 * i + c];
          d[3 * j + c] = bank.dir[3 * i + c];
        }
        const auto& e = excl[pend[j]];
        ids.insert(ids.end(), e.begin(), e.end());
        off[j + 1] = (int32_t)ids.size();
      }
      if (ids.empty()) ids.push_back(0);
      rt.check(xdgcu_ray_fire(ctx, ipc_surface_tree, nullptr, (int64_t)m, o.data(), d.data(),
                              nullptr, XDGCU_EXITING, off.data(), ids.data(), t.data(),
                              surf.data(), face.data(), nullptr, prec, nullptr),
               "ray_fire");
      std::vector<size_t> hitters;
      std::vector<double> q;
      for (size_t j = 0; j < m; ++j) {
        if (surf[j] == ID_NONE) continue;  // no re-entry point: the particle ends
        const size_t i = out[pend[j]];
        for (int c = 0; c < 3; ++c) bank.pos[3 * i + c] = bank.pos[3 * i + c] + bank.dir[3 * i + c] * t[j];
        bank.distance[i] = bank.distance[i] + t[j];
        excl[pend[j]].push_back(face[j]);  // ray_fire appends the hit face
        for (int c = 0; c < 3; ++c) q.push_back(bank.pos[3 * i + c] + bank.dir[3 * i + c] * TINY_BIT);
        hitters.push_back(pend[j]);
      }
      if (hitters.empty()) break;
      std::vector<int32_t> eid(hitters.size()), eidx(hitters.size());
      rt.check(xdgcu_find_element(ctx, gtree, nullptr, (int64_t)hitters.size(), q.data(),
                                  eid.data(), eidx.data(), nullptr, prec, nullptr),
               "find_element");
      std::vector<size_t> next;
      for (size_t j = 0; j < hitters.size(); ++j) {
        found[hitters[j]] = eidx[j];
        if (eidx[j] < 0 && excl[hitters[j]].size() < 64) next.push_back(hitters[j]);
      }
      pend.swap(next);
    }
    bool any = false;
    for (size_t k = 0; k < out.size(); ++k) {
      idx[out[k]] = found[k];
      if (found[k] < 0) ended[out[k]] = 1;
      else any = true;
    }
    if (!any) break;
  }
  for (size_t i = 0; i < n; ++i) bank.cell[i] = rt.tet_id(idx[i]);
}

// ---------------------------------------------------------------------------
// particle_sim tool
// ---------------------------------------------------------------------------

void simulate_particles(CudaRayTracer& rt, const MeshManager& mm,
                        const std::map<MeshID, TreeID>& volume_trees, bool ipc_graveyard,
                        ParticleBank& bank, double mfp, int32_t max_events,
                        std::map<MeshID, double>* cell_tracks, int32_t history_cap) {
  xdgcu_ctx* ctx = rt.context();
  // boundary conditions (particle_sim.h:80-118 reads them per crossing)
  std::vector<int32_t> sids, bcs;
  for (MeshID s : mm.surfaces()) {
    const std::string v = mm.get_surface_property(s, PropertyType::BOUNDARY_CONDITION).value;
    sids.push_back(s);
    bcs.push_back(v == "reflecting" || v == "reflective" ? XDGCU_BC_REFLECTING
                  : v == "vacuum"                         ? XDGCU_BC_VACUUM
                                                          : XDGCU_BC_TRANSMISSION);
  }
  rt.check(xdgcu_set_surface_boundary(ctx, (int32_t)sids.size(), sids.data(), bcs.data()),
           "set_surface_boundary");
  const size_t n = bank.size();
  std::map<TreeID, MeshID> volume_of;
  for (const auto& vt : volume_trees) volume_of[vt.second] = vt.first;
  std::vector<int32_t> tree(n);
  for (size_t i = 0; i < n; ++i) tree[i] = bank.cell[i] == ID_NONE ? -1 : volume_trees.at(bank.cell[i]);
  const TreeID grave = ipc_graveyard ? volume_trees.at(mm.implicit_complement()) : 0;
  std::vector<int32_t> hist(n * (size_t)history_cap, 0), hc(n, 0);
  const int32_t n_trees = xdgcu_num_surface_trees(ctx);
  std::vector<double> tally(cell_tracks ? (size_t)n_trees + 1 : 0, 0.0);
  rt.check(xdgcu_transport_surfaces(ctx, (int64_t)n, tree.data(), bank.pos.data(),
                                    bank.dir.data(), bank.rng.data(), mfp, max_events, grave,
                                    history_cap, hist.data(), hc.data(), bank.distance.data(),
                                    bank.events.data(), cell_tracks ? tally.data() : nullptr,
                                    bank.status.data(), rt.precision(), nullptr),
           "transport_surfaces");
  for (size_t i = 0; i < n; ++i) {
    auto it = volume_of.find(tree[i]);
    bank.cell[i] = it == volume_of.end() ? ID_NONE : it->second;
  }
  if (cell_tracks)
    for (const auto& vt : volume_trees) (*cell_tracks)[vt.first] += tally[vt.second];
}

// ---------------------------------------------------------------------------
// XDG::segments over the whole model
// ---------------------------------------------------------------------------

TrackSegments track_segments(CudaRayTracer& rt, const MeshManager& mm, TreeID ipc_surface_tree,
                             size_t n, const double* starts, const double* ends, int max_rounds) {
  xdgcu_ctx* ctx = rt.context();
  const int prec = rt.precision();
  // MeshManager::get_boundary_face_element of every surface face, as tet
  // indices of the engine's mesh
  std::vector<int32_t> faces, elems;
  for (MeshID s : mm.surfaces())
    for (MeshID f : mm.get_surface_faces(s)) {
      const MeshID be = mm.get_boundary_face_element(f);
      faces.push_back(f);
      elems.push_back(be == ID_NONE ? -1 : rt.tet_index(be));
    }
  rt.check(xdgcu_set_boundary_face_elements(ctx, (int64_t)faces.size(), faces.data(), elems.data()),
           "set_boundary_face_elements");
  // every round of every track in one call; sized again when the first
  // guess of the output size is too small
  TrackSegments out;
  out.offsets.assign(n + 1, 0);
  int64_t cap = std::max<int64_t>(1024, 64 * (int64_t)n);
  for (int attempt = 0; attempt < 2; ++attempt) {
    out.element.resize(cap);
    out.length.resize(cap);
    rt.check(xdgcu_segments_global(ctx, ipc_surface_tree, rt.global_element_tree_id(), (int64_t)n,
                                   starts, ends, 4096, max_rounds, cap, out.element.data(),
                                   out.length.data(), out.offsets.data(), nullptr, prec, nullptr),
             "segments_global");
    if (out.offsets[n] <= cap) break;
    cap = out.offsets[n];
  }
  out.element.resize(out.offsets[n]);
  out.length.resize(out.offsets[n]);
  return out;
}

// ---------------------------------------------------------------------------
// overlap_check tool
// ---------------------------------------------------------------------------

std::map<std::set<MeshID>, Position> check_overlaps(CudaRayTracer& rt, const MeshManager& mm,
                                                    const std::map<MeshID, TreeID>& volume_trees,
                                                    bool check_edges, int64_t max_batch) {
  xdgcu_ctx* ctx = rt.context();
  const int prec = rt.precision();
  std::map<std::set<MeshID>, Position> found;
  const std::vector<MeshID>& vols = mm.volumes();
  std::vector<int32_t> trees;
  for (MeshID v : vols) trees.push_back(volume_trees.at(v));
  const int64_t nv = (int64_t)vols.size();

  // overlap.cpp:9-60 for every face vertex (:74-85), in surface order
  std::vector<Vertex> verts;
  for (MeshID s : mm.surfaces())
    for (MeshID f : mm.get_surface_faces(s))
      for (const Vertex& v : mm.face_vertices(f)) verts.push_back(v);
  const Direction d = normalized({0.1, 0.1, 0.1});
  const Direction d2 = -d;
  const double bump = 1e-9;
  const int64_t step = std::max<int64_t>(1, max_batch / std::max<int64_t>(1, 2 * nv));
  for (int64_t k0 = 0; k0 < (int64_t)verts.size(); k0 += step) {
    const int64_t k1 = std::min<int64_t>((int64_t)verts.size(), k0 + step);
    const int64_t m = 2 * (k1 - k0);
    std::vector<double> pts(3 * m), dirs(3 * m);
    for (int64_t k = k0; k < k1; ++k) {
      const Position loc1 = verts[k] + d * bump;           // loc += dir * bump
      const Position loc2 = loc1 + (d2 * 2.0) * bump;      // loc += dir * 2.0 * bump
      const int64_t j = 2 * (k - k0);
      for (int c = 0; c < 3; ++c) {
        pts[3 * j + c] = loc1[c];
        pts[3 * (j + 1) + c] = loc2[c];
        dirs[3 * j + c] = d[c];
        dirs[3 * (j + 1) + c] = d2[c];
      }
    }
    std::vector<uint8_t> inside((size_t)(m * nv));
    rt.check(xdgcu_point_in_volumes(ctx, m, pts.data(), dirs.data(), (int32_t)nv, trees.data(),
                                    inside.data(), nullptr, prec, nullptr),
             "point_in_volumes");
    for (int64_t j = 0; j < m; ++j) {
      std::set<MeshID> key;
      for (int64_t v = 0; v < nv; ++v)
        if (inside[j * nv + v]) key.insert(vols[v]);
      if (key.size() > 1 && !found.count(key))
        found[key] = {pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]};
    }
  }
  if (!check_edges) return found;

  // overlap.cpp:139-176, 213-230 and check_along_edge
  for (MeshID s : mm.surfaces()) {
    const auto parents = mm.get_parent_volumes(s);
    std::vector<MeshID> check;
    for (MeshID v : vols)
      if (v != parents.first && v != parents.second) check.push_back(v);
    if (check.empty()) continue;
    std::vector<int32_t> ctrees;
    for (MeshID v : check) ctrees.push_back(volume_trees.at(v));
    std::vector<double> o, dd, len;
    for (MeshID f : mm.get_surface_faces(s)) {
      const std::array<Vertex, 3> tri = mm.face_vertices(f);
      for (size_t k = 0; k < 3; ++k) {
        const Vertex& v1 = tri[k];
        const Vertex& v2 = tri[(k + 1) % 3];
        Direction dir = v2 - v1;
        const double ln = dir.length();
        dir = {dir.x / ln, dir.y / ln, dir.z / ln};  // dir /= edgeLength
        o.insert(o.end(), {v1.x, v1.y, v1.z});
        dd.insert(dd.end(), {dir.x, dir.y, dir.z});
        len.push_back(ln);
      }
    }
    const int64_t ne = (int64_t)len.size(), nc = (int64_t)check.size();
    const int64_t estep = std::max<int64_t>(1, max_batch / nc);
    for (int64_t e0 = 0; e0 < ne; e0 += estep) {
      const int64_t e1 = std::min(ne, e0 + estep), m = (e1 - e0) * nc;
      std::vector<double> ro(3 * m), rd(3 * m), rl(m), t(m);
      std::vector<int32_t> rt_ids(m), surf(m), face(m);
      for (int64_t e = e0; e < e1; ++e)
        for (int64_t c = 0; c < nc; ++c) {
          const int64_t r = (e - e0) * nc + c;
          for (int a = 0; a < 3; ++a) {
            ro[3 * r + a] = o[3 * e + a];
            rd[3 * r + a] = dd[3 * e + a];
          }
          rl[r] = len[e];
          rt_ids[r] = ctrees[c];
        }
      rt.check(xdgcu_ray_fire(ctx, 0, rt_ids.data(), m, ro.data(), rd.data(), rl.data(),
                              XDGCU_EXITING, nullptr, nullptr, t.data(), surf.data(), face.data(),
                              nullptr, prec, nullptr),
               "ray_fire");
      for (int64_t e = e0; e < e1; ++e)
        for (int64_t c = 0; c < nc; ++c) {  // the first volume with a hit
          const int64_t r = (e - e0) * nc + c;
          if (surf[r] == ID_NONE) continue;
          const std::set<MeshID> key = {mm.get_parent_volumes(surf[r]).first, parents.first};
          if (!found.count(key))
            found[key] = {ro[3 * r] + t[r] * rd[3 * r], ro[3 * r + 1] + t[r] * rd[3 * r + 1],
                          ro[3 * r + 2] + t[r] * rd[3 * r + 2]};
          break;
        }
    }
  }
  return found;
}

}  // namespace xdg
