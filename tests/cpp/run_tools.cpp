// Runs one of the C++ tool loops (xdg_gb300/cpp/cuda_tools.*) on a model and
// particle state read from binary files, and writes the results, so that
// tests/test_cpp_tools.py can compare them with the Python engine's and the
// oracle's.  Usage: run_tools MODEL JOB OUT
//
// MODEL (little-endian int32 / float64):
//   n_surfaces; per surface: id, forward volume, reverse volume, n_faces,
//     n_faces face ids, n_faces x 9 coordinates (the face's vertices in order)
//   n_volumes, the volume ids, the implicit complement
//   n_bc, (surface id, 0 transmission / 1 vacuum / 2 reflecting) pairs
//   has_tets; if so: n_vertices, coordinates, n_tets, connectivity (4 per
//     tet), adjacency (4 tet indices per tet, -1 on the boundary, MOAB face
//     order), element ids, per volume (in volume order) its tet count and
//     tet indices, and n_bfe, the tet index behind each face id
//     0 .. n_bfe-1 (-1: none; MeshManager::get_boundary_face_element)
// JOB: job (1 walk_particles, 2 simulate_particles, 3 check_overlaps,
//   4 track_segments), precision; for 1 and 2: n, n cells (element / volume
//   ids), n x 3 positions, n x 3 directions, n stream states (uint64), mfp,
//   max_events, and for 2 the graveyard flag; for 3 the check_edges flag;
//   for 4: n, n x 3 starts, n x 3 ends.
// OUT: for 1 and 2 the bank (cells, positions, directions, streams,
//   distances, events, statuses); for 3 the number of sets, then per set its
//   size, the volume ids and the location; for 4 the n + 1 offsets (int64),
//   the segments' element ids and lengths.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "cuda_tools.h"

using namespace xdg;

namespace {

struct Reader {
  FILE* f;
  explicit Reader(const char* path) : f(std::fopen(path, "rb")) {
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  }
  ~Reader() { std::fclose(f); }
  template <typename T>
  T get() {
    T v;
    if (std::fread(&v, sizeof v, 1, f) != 1) throw std::runtime_error("short read");
    return v;
  }
  template <typename T>
  std::vector<T> vec(size_t n) {
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short read");
    return v;
  }
};

struct Writer {
  FILE* f;
  explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  }
  ~Writer() { std::fclose(f); }
  template <typename T>
  void put(const T& v) { std::fwrite(&v, sizeof v, 1, f); }
  template <typename T>
  void vec(const std::vector<T>& v) { std::fwrite(v.data(), sizeof(T), v.size(), f); }
};

const int MOAB_FACES[4][3] = {{0, 1, 3}, {1, 2, 3}, {2, 0, 3}, {0, 2, 1}};

class FileMesh : public MeshManager {
 public:
  explicit FileMesh(Reader& r) {
    const int32_t ns = r.get<int32_t>();
    for (int32_t k = 0; k < ns; ++k) {
      const int32_t id = r.get<int32_t>(), fwd = r.get<int32_t>(), rev = r.get<int32_t>();
      const int32_t nf = r.get<int32_t>();
      const std::vector<int32_t> faces = r.vec<int32_t>(nf);
      const std::vector<double> xyz = r.vec<double>(9 * (size_t)nf);
      surfaces_.push_back(id);
      senses_[id] = {fwd, rev};
      faces_[id] = faces;
      for (int32_t j = 0; j < nf; ++j)
        for (int v = 0; v < 3; ++v)
          face_xyz_[faces[j]][v] = {xyz[9 * j + 3 * v], xyz[9 * j + 3 * v + 1],
                                    xyz[9 * j + 3 * v + 2]};
    }
    const int32_t nv = r.get<int32_t>();
    volumes_ = r.vec<int32_t>(nv);
    implicit_complement_ = r.get<int32_t>();
    const int32_t nbc = r.get<int32_t>();
    for (int32_t k = 0; k < nbc; ++k) {
      const int32_t s = r.get<int32_t>(), code = r.get<int32_t>();
      surface_metadata_[{s, PropertyType::BOUNDARY_CONDITION}] = {
          PropertyType::BOUNDARY_CONDITION,
          code == 1 ? "vacuum" : (code == 2 ? "reflecting" : "transmission")};
    }
    if (r.get<int32_t>()) {
      const int32_t nvert = r.get<int32_t>();
      verts_ = r.vec<double>(3 * (size_t)nvert);
      const int32_t nt = r.get<int32_t>();
      conn_ = r.vec<int32_t>(4 * (size_t)nt);
      adj_ = r.vec<int32_t>(4 * (size_t)nt);
      ids_ = r.vec<int32_t>(nt);
      for (int32_t t = 0; t < nt; ++t) index_[ids_[t]] = t;
      for (int32_t v : volumes_) {
        const int32_t c = r.get<int32_t>();
        const std::vector<int32_t> tets = r.vec<int32_t>(c);
        for (int32_t t : tets) elements_[v].push_back(ids_[t]);
      }
      const int32_t nb = r.get<int32_t>();
      bfe_ = r.vec<int32_t>(nb);
    }
  }
  std::vector<MeshID> get_volume_surfaces(MeshID v) const override {
    std::vector<MeshID> out;
    for (MeshID s : surfaces_) {
      const auto& sn = senses_.at(s);
      if (sn.first == v || sn.second == v) out.push_back(s);
    }
    return out;
  }
  std::vector<MeshID> get_surface_faces(MeshID s) const override { return faces_.at(s); }
  std::array<Vertex, 3> face_vertices(MeshID f) const override { return face_xyz_.at(f); }
  std::pair<MeshID, MeshID> surface_senses(MeshID s) const override { return senses_.at(s); }
  std::vector<MeshID> get_volume_elements(MeshID v) const override {
    auto it = elements_.find(v);
    return it == elements_.end() ? std::vector<MeshID>{} : it->second;
  }
  std::vector<Vertex> element_vertices(MeshID e) const override {
    std::vector<Vertex> out;
    for (MeshID v : element_connectivity(e)) out.push_back(vertex_coordinates(v));
    return out;
  }
  std::vector<MeshID> element_connectivity(MeshID e) const override {
    const int32_t t = index_.at(e);
    return {conn_[4 * t], conn_[4 * t + 1], conn_[4 * t + 2], conn_[4 * t + 3]};
  }
  Vertex vertex_coordinates(MeshID v) const override {
    return {verts_[3 * v], verts_[3 * v + 1], verts_[3 * v + 2]};
  }
  MeshID adjacent_element(MeshID e, int face) const override {
    const int32_t nb = adj_[4 * index_.at(e) + face];
    return nb < 0 ? ID_NONE : ids_[nb];
  }
  MeshID get_boundary_face_element(MeshID face) const override {
    if (face < 0 || face >= (MeshID)bfe_.size() || bfe_[face] < 0) return ID_NONE;
    return ids_[bfe_[face]];
  }
  MeshLibrary mesh_library() const override { return MeshLibrary::MOAB; }

 private:
  std::map<MeshID, std::pair<MeshID, MeshID>> senses_;
  std::map<MeshID, std::vector<MeshID>> faces_;
  std::map<MeshID, std::array<Vertex, 3>> face_xyz_;
  std::vector<double> verts_;
  std::vector<int32_t> conn_, adj_, ids_, bfe_;
  std::map<MeshID, int32_t> index_;
  std::map<MeshID, std::vector<MeshID>> elements_;
};

struct MoabFaces : ElementFaceAccessor {
  MoabFaces(const MeshManager* mm, MeshID e) : ElementFaceAccessor(e), mm_(mm) {}
  std::array<Vertex, 3> face_vertices(int i) const override {
    const std::vector<Vertex> v = mm_->element_vertices(element_);
    return {v[MOAB_FACES[i][0]], v[MOAB_FACES[i][1]], v[MOAB_FACES[i][2]]};
  }
  const MeshManager* mm_;
};

}  // namespace

std::shared_ptr<ElementFaceAccessor> ElementFaceAccessor::create(const MeshManager* mm,
                                                                 MeshID element) {
  return std::make_shared<MoabFaces>(mm, element);
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s MODEL JOB OUT\n", argv[0]);
    return 2;
  }
  try {
    Reader rm(argv[1]);
    auto mm = std::make_shared<FileMesh>(rm);
    Reader rj(argv[2]);
    const int32_t job = rj.get<int32_t>(), prec = rj.get<int32_t>();
    CudaRayTracer rt(0, prec);
    std::map<MeshID, TreeID> volume_trees;
    for (MeshID v : mm->volumes()) volume_trees[v] = rt.register_volume(mm, v).first;
    rt.create_global_element_tree();
    rt.create_global_surface_tree();
    Writer w(argv[3]);
    if (job == 1 || job == 2) {
      const int32_t n = rj.get<int32_t>();
      ParticleBank b;
      b.resize(n);
      b.cell = rj.vec<int32_t>(n);
      b.pos = rj.vec<double>(3 * (size_t)n);
      b.dir = rj.vec<double>(3 * (size_t)n);
      b.rng = rj.vec<uint64_t>(n);
      const double mfp = rj.get<double>();
      const int32_t max_events = rj.get<int32_t>();
      if (job == 1) {
        walk_particles(rt, volume_trees.at(mm->implicit_complement()), b, mfp, max_events);
      } else {
        const int32_t grave = rj.get<int32_t>();
        simulate_particles(rt, *mm, volume_trees, grave != 0, b, mfp, max_events);
      }
      w.vec(b.cell);
      w.vec(b.pos);
      w.vec(b.dir);
      w.vec(b.rng);
      w.vec(b.distance);
      w.vec(b.events);
      w.vec(b.status);
    } else if (job == 3) {
      const int32_t edges = rj.get<int32_t>();
      const auto found = check_overlaps(rt, *mm, volume_trees, edges != 0);
      w.put((int32_t)found.size());
      for (const auto& kv : found) {
        w.put((int32_t)kv.first.size());
        for (MeshID v : kv.first) w.put((int32_t)v);
        w.put(kv.second.x);
        w.put(kv.second.y);
        w.put(kv.second.z);
      }
    } else if (job == 4) {
      const int32_t n = rj.get<int32_t>();
      const std::vector<double> a = rj.vec<double>(3 * (size_t)n);
      const std::vector<double> b = rj.vec<double>(3 * (size_t)n);
      const TrackSegments s = track_segments(rt, *mm, volume_trees.at(mm->implicit_complement()),
                                             (size_t)n, a.data(), b.data());
      w.vec(s.offsets);
      w.vec(s.element);
      w.vec(s.length);
    } else {
      std::fprintf(stderr, "unknown job %d\n", job);
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
