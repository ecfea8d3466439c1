// pybind11 module `visacd`: the reference's Python surface (lib/bindings.cpp:14-70)
// — Mesh, VecArray3d, VecArray3i, MeshList, Config, make_vecarray3i, set_seed,
// config (a reference to the process-wide configuration), ProcessResult,
// process — plus underscore-prefixed helpers used by this project's tests and
// benchmarks.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <pybind11/stl_bind.h>

#include "geometry.hpp"
#include "gpu_bridge.hpp"
#include "process.hpp"
#include "visacd_gpu.h"

namespace py = pybind11;
using namespace visacd;

PYBIND11_MAKE_OPAQUE(std::vector<std::array<double, 3>>);
PYBIND11_MAKE_OPAQUE(std::vector<std::array<int, 3>>);
PYBIND11_MAKE_OPAQUE(visacd::MeshList);

namespace {

py::array_t<double> verts_to_np(const std::vector<Vec3>& v) {
  py::array_t<double> a({(py::ssize_t)v.size(), (py::ssize_t)3});
  auto r = a.mutable_unchecked<2>();
  for (size_t i = 0; i < v.size(); ++i)
    for (int k = 0; k < 3; ++k) r(i, k) = v[i][k];
  return a;
}

py::array_t<int> tris_to_np(const std::vector<Tri>& t) {
  py::array_t<int> a({(py::ssize_t)t.size(), (py::ssize_t)3});
  auto r = a.mutable_unchecked<2>();
  for (size_t i = 0; i < t.size(); ++i)
    for (int k = 0; k < 3; ++k) r(i, k) = t[i][k];
  return a;
}

Mesh np_to_mesh(py::array_t<double, py::array::c_style | py::array::forcecast> v,
                py::array_t<int, py::array::c_style | py::array::forcecast> t) {
  Mesh m;
  auto rv = v.unchecked<2>();
  auto rt = t.unchecked<2>();
  m.vertices.resize(rv.shape(0));
  for (py::ssize_t i = 0; i < rv.shape(0); ++i) m.vertices[i] = {rv(i, 0), rv(i, 1), rv(i, 2)};
  m.triangles.resize(rt.shape(0));
  for (py::ssize_t i = 0; i < rt.shape(0); ++i) m.triangles[i] = {rt(i, 0), rt(i, 1), rt(i, 2)};
  return m;
}

py::dict mesh_dict(const Mesh& m) {
  py::dict d;
  d["vertices"] = verts_to_np(m.vertices);
  d["triangles"] = tris_to_np(m.triangles);
  py::array_t<uint8_t> nw((py::ssize_t)m.is_new.size());
  for (size_t i = 0; i < m.is_new.size(); ++i) nw.mutable_at(i) = m.is_new[i] ? 1 : 0;
  d["is_new"] = nw;
  py::array_t<uint32_t> e({(py::ssize_t)m.intersecting_edges.size(), (py::ssize_t)2});
  for (size_t i = 0; i < m.intersecting_edges.size(); ++i) {
    e.mutable_at(i, 0) = m.intersecting_edges[i].first;
    e.mutable_at(i, 1) = m.intersecting_edges[i].second;
  }
  d["edges"] = e;
  return d;
}

}  // namespace

PYBIND11_MODULE(visacd, m) {
  py::bind_vector<std::vector<std::array<double, 3>>>(m, "VecArray3d");
  py::bind_vector<std::vector<std::array<int, 3>>>(m, "VecArray3i");

  py::class_<Mesh>(m, "Mesh")
      .def(py::init<>())
      .def_readwrite("vertices", &Mesh::vertices)
      .def_readwrite("triangles", &Mesh::triangles)
      // Additions: zero-copy numpy views of the mesh's own storage (N x 3
      // float64 / int32). A view keeps the mesh alive and stays valid until
      // the mesh's vertices / triangles are reassigned or resized.
      .def("vertex_array",
           [](py::object self) {
             Mesh& mm = self.cast<Mesh&>();
             return py::array_t<double>({(py::ssize_t)mm.vertices.size(), (py::ssize_t)3},
                                        {(py::ssize_t)sizeof(Vec3), (py::ssize_t)sizeof(double)},
                                        reinterpret_cast<const double*>(mm.vertices.data()), self);
           })
      .def("triangle_array", [](py::object self) {
        Mesh& mm = self.cast<Mesh&>();
        return py::array_t<int>({(py::ssize_t)mm.triangles.size(), (py::ssize_t)3},
                                {(py::ssize_t)sizeof(Tri), (py::ssize_t)sizeof(int)},
                                reinterpret_cast<const int*>(mm.triangles.data()), self);
      });

  py::bind_vector<MeshList>(m, "MeshList");

  py::class_<Config>(m, "Config")
      .def(py::init<>())
      .def_readwrite("return_parts", &Config::return_parts)
      .def_readwrite("score_mode", &Config::score_mode)
      .def_readwrite("flat_surface_min_area", &Config::flat_surface_min_area)
      .def_readwrite("use_flat_surfaces", &Config::use_flat_surfaces)
      .def_readwrite("flat_surface_k", &Config::flat_surface_k)
      .def_readwrite("use_merging", &Config::use_merging)
      .def_readwrite("verbose", &Config::verbose)
      .def_readwrite("plane_proposer", &Config::plane_proposer)
      .def_readwrite("proposer_weights", &Config::proposer_weights)
      .def_readwrite("proposer_probe_planes", &Config::proposer_probe_planes)
      .def_readwrite("proposer_refine", &Config::proposer_refine)
      .def_readwrite("proposer_tolerance", &Config::proposer_tolerance);

  m.def("make_vecarray3i", [](py::array_t<int, py::array::c_style | py::array::forcecast> a) {
    auto buf = a.request();
    std::vector<std::array<int, 3>> out;
    const int* p = static_cast<const int*>(buf.ptr);
    const py::ssize_t rows = buf.ndim >= 1 ? buf.shape[0] : 0;
    out.reserve(rows);
    for (py::ssize_t i = 0; i < rows; ++i) out.push_back({p[3 * i], p[3 * i + 1], p[3 * i + 2]});
    return out;
  });

  m.def("set_seed", &set_seed, py::arg("seed"));
  // Test hook (not in the reference's surface): route stages through the host
  // restatements their GPU kernels are checked against. Arguments left at
  // None keep their setting; returns the settings after the call.
  m.def(
      "_checker_hooks",
      [](py::object clip, py::object concavity, py::object remesh, py::object merge, py::object hull) {
        CheckerHooks& h = checker_hooks();
        if (!clip.is_none()) h.host_clip = clip.cast<bool>();
        if (!concavity.is_none()) h.host_concavity = concavity.cast<bool>();
        if (!remesh.is_none()) h.host_remesh = remesh.cast<bool>();
        if (!merge.is_none()) h.host_merge = merge.cast<bool>();
        if (!hull.is_none()) h.host_hull = hull.cast<bool>();
        py::dict d;
        d["host_clip"] = h.host_clip;
        d["host_concavity"] = h.host_concavity;
        d["host_remesh"] = h.host_remesh;
        d["host_merge"] = h.host_merge;
        d["host_hull"] = h.host_hull;
        return d;
      },
      py::arg("host_clip") = py::none(), py::arg("host_concavity") = py::none(),
      py::arg("host_remesh") = py::none(), py::arg("host_merge") = py::none(),
      py::arg("host_hull") = py::none());
  // Test hook: record every visibility call of process() (the part with its
  // is_new mask and the edges found, and its cage); reading clears the record.
  m.def("_record_visibility", [](bool on) {
    checker_hooks().record_visibility = on;
    recorded_visibility().clear();
    recorded_splits().clear();
  });
  m.def("_recorded_splits", []() {
    py::list out;
    for (const auto& r : recorded_splits()) out.append(py::make_tuple(r[0], r[1], r[2], r[3], r[4]));
    recorded_splits().clear();
    return out;
  });
  m.def("_recorded_visibility", []() {
    py::list out;
    for (const auto& r : recorded_visibility()) {
      py::dict d;
      d["part"] = mesh_dict(r.part);
      d["cage"] = mesh_dict(r.cage);
      out.append(d);
    }
    recorded_visibility().clear();
    return out;
  });
  m.attr("config") = py::cast(&config(), py::return_value_policy::reference);
  // The trained proposer ships next to this module (proposer_weights.bin).
  if (config().proposer_weights.empty()) {
    try {
      auto os_path = py::module_::import("os.path");
      py::object here = os_path.attr("dirname")(py::module_::import("visacd_gb300").attr("__file__"));
      config().proposer_weights = py::cast<std::string>(os_path.attr("join")(here, "proposer_weights.bin"));
    } catch (const py::error_already_set&) {
    }
  }

  py::class_<ProcessResult>(m, "ProcessResult")
      .def_readwrite("parts", &ProcessResult::parts)
      .def_readwrite("concavity", &ProcessResult::concavity)
      .def_readwrite("num_parts", &ProcessResult::num_parts);

  m.def("process", &process, py::arg("mesh"), py::arg("concavity"), py::arg("num_parts"),
        py::call_guard<py::gil_scoped_release>());
  // Addition: many meshes at once (see process.hpp).
  m.def("process_batch", &process_batch, py::arg("meshes"), py::arg("concavity"), py::arg("num_parts"),
        py::arg("seeds"), py::arg("threads") = 0, py::call_guard<py::gil_scoped_release>());

  // ---- helpers for tests and benchmarks (not part of the reference surface) --
  m.def("_stage_times", []() {
    const auto& t = last_stage_times();
    py::dict d;
    d["preprocess_ms"] = t.preprocess;
    d["visibility_ms"] = t.visibility;
    d["scoring_ms"] = t.scoring;
    d["clip_ms"] = t.clip;
    d["concavity_ms"] = t.concavity;
    d["cages_ms"] = t.cages;
    d["hulls_ms"] = t.hulls;
    d["total_ms"] = t.total;
    d["iterations"] = t.iterations;
    const auto& c = gpu::counters();
    d["vis_calls"] = c.vis_calls;
    d["vis_pairs"] = c.vis_pairs;
    d["vis_edges"] = c.vis_edges;
    d["score_calls"] = c.score_calls;
    d["plane_edge_pairs"] = c.plane_edge_pairs;
    d["lp_calls"] = c.lp_calls;
    d["lp_fallbacks"] = c.lp_fallbacks;
    d["lp_ms"] = c.lp_ms;
    d["vis_ms"] = c.vis_ms;
    d["score_ms"] = c.score_ms;
    const auto& ct = concavity_times();
    d["conc_sample_ms"] = ct.sample_ms;
    d["conc_hausdorff_ms"] = ct.hausdorff_ms;
    d["conc_hull_ms"] = ct.hull_ms;
    d["conc_samples"] = ct.samples;
    d["conc_calls"] = ct.calls;
    return d;
  });
  m.def("_gpu_timing", [](bool on) {
    visacd_ctx_set_timing(gpu::context(), on ? 1 : 0);
    visacd_ctx_reset_times(gpu::context());
  });
  m.def("_gpu_kernel_times", []() {
    const char* names[96];
    double ms[96];
    int64_t launches[96];
    int n = 0;
    py::dict d;
    if (visacd_ctx_kernel_times(gpu::context(), names, ms, launches, 96, &n) == VISACD_OK)
      for (int i = 0; i < n; ++i)
        if (launches[i]) d[names[i]] = py::make_tuple(ms[i], launches[i]);
    return d;
  });
  m.def("_reset_counters", []() {
    gpu::counters() = gpu::Counters();
    concavity_times() = ConcavityTimes();
  });
  m.def("_manifold_preprocess", [](py::array_t<double> v, py::array_t<int> t, double scale, double level) {
    Mesh mm = np_to_mesh(v, t);
    manifold_preprocess_host(mm, scale, level);
    return mesh_dict(mm);
  });
  m.def("_manifold_preprocess_gpu", [](py::array_t<double> v, py::array_t<int> t, double scale, double level) {
    Mesh mm = np_to_mesh(v, t);
    gpu::sdf_remesh(mm, scale, level);
    return mesh_dict(mm);
  });
  m.def(
      "_convex_hull",
      [](py::array_t<double> v, bool fix_normals) {
        Mesh tmp = np_to_mesh(v, py::array_t<int>(std::vector<py::ssize_t>{0, 3}));
        return mesh_dict(convex_hull(tmp.vertices, fix_normals));
      },
      py::arg("v"), py::arg("fix_normals") = true);
  m.def("_clip", [](py::array_t<double> v, py::array_t<int> t, std::array<double, 4> pl) {
    Mesh mm = np_to_mesh(v, t);
    std::vector<int> m1, m2;
    MeshList out = clip(mm, Plane(pl[0], pl[1], pl[2], pl[3]), m1, m2);
    py::list parts;
    for (const auto& p : out) parts.append(mesh_dict(p));
    return py::make_tuple(parts, m1, m2);
  });
  m.def("_clip_gpu", [](py::array_t<double> v, py::array_t<int> t, std::array<double, 4> pl) {
    Mesh mm = np_to_mesh(v, t);
    std::vector<int> m1, m2;
    MeshList out = gpu::clip(mm, Plane(pl[0], pl[1], pl[2], pl[3]), m1, m2);
    py::list parts;
    for (const auto& p : out) parts.append(mesh_dict(p));
    return py::make_tuple(parts, m1, m2);
  });
  m.def("_candidate_planes", [](py::array_t<double> v, py::array_t<uint32_t> e, int num) {
    Mesh mm = np_to_mesh(v, py::array_t<int>(std::vector<py::ssize_t>{0, 3}));
    auto re = e.unchecked<2>();
    std::vector<Edge> edges(re.shape(0));
    for (py::ssize_t i = 0; i < re.shape(0); ++i) edges[i] = {re(i, 0), re(i, 1)};
    auto planes = get_candidate_planes(mm.vertices, edges, num);
    py::array_t<double> out({(py::ssize_t)planes.size(), (py::ssize_t)4});
    for (size_t i = 0; i < planes.size(); ++i) {
      out.mutable_at(i, 0) = planes[i].a;
      out.mutable_at(i, 1) = planes[i].b;
      out.mutable_at(i, 2) = planes[i].c;
      out.mutable_at(i, 3) = planes[i].d;
    }
    return out;
  });
  m.def("_extract_surfaces", [](py::array_t<double> v, py::array_t<int> t, double min_area) {
    Mesh mm = np_to_mesh(v, t);
    auto s = extract_surfaces(mm, min_area);
    py::list out;
    for (const auto& x : s) out.append(py::make_tuple(x.area, std::array<double, 4>{x.plane.a, x.plane.b, x.plane.c, x.plane.d}, x.triangle_ids));
    return out;
  });
  m.def("_compute_h", [](py::array_t<double> v, py::array_t<int> t, double k, unsigned res) {
    Mesh mm = np_to_mesh(v, t);
    Mesh h = convex_hull(mm.vertices, true);
    return compute_h(mm, h, k, res);
  });
  m.def("_compute_hb", [](py::array_t<double> v, py::array_t<int> t, py::array_t<double> hv, py::array_t<int> ht, unsigned res) {
    return compute_hb(np_to_mesh(v, t), np_to_mesh(hv, ht), res);
  });
  m.def("_refine_proposals", [](py::array_t<double> v, py::array_t<uint32_t> edges, py::array_t<double> planes,
                                int per) {
    Mesh mm;
    auto vv = v.unchecked<2>();
    for (py::ssize_t i = 0; i < vv.shape(0); ++i) mm.vertices.push_back({vv(i, 0), vv(i, 1), vv(i, 2)});
    auto ee = edges.unchecked<2>();
    for (py::ssize_t i = 0; i < ee.shape(0); ++i) mm.intersecting_edges.push_back({ee(i, 0), ee(i, 1)});
    auto pp = planes.unchecked<2>();
    std::vector<Plane> prop;
    for (py::ssize_t i = 0; i < pp.shape(0); ++i) prop.emplace_back(pp(i, 0), pp(i, 1), pp(i, 2), pp(i, 3));
    const auto out = refine_proposals(mm, prop, per);
    py::array_t<double> r({(py::ssize_t)out.size(), (py::ssize_t)4});
    for (size_t i = 0; i < out.size(); ++i) {
      r.mutable_at(i, 0) = out[i].a;
      r.mutable_at(i, 1) = out[i].b;
      r.mutable_at(i, 2) = out[i].c;
      r.mutable_at(i, 3) = out[i].d;
    }
    return r;
  });
  m.def("_engine_next", [](int n) {
    std::vector<uint32_t> w((size_t)std::max(n, 0));
    random_engine().fill(w.data(), w.size());
    return py::array_t<uint32_t>(w.size(), w.data());
  });
  m.def("_sample_points", [](py::array_t<double> v, py::array_t<int> t, unsigned res) {
    std::vector<Vec3> x;
    std::vector<int> ids;
    extract_point_set(np_to_mesh(v, t), x, ids, res, 1, true);
    return py::make_tuple(verts_to_np(x), py::array_t<int>(ids.size(), ids.data()));
  });
  m.def("_mesh_dist", [](py::array_t<double> a, py::array_t<double> b) {
    Mesh ma = np_to_mesh(a, py::array_t<int>(std::vector<py::ssize_t>{0, 3}));
    Mesh mb = np_to_mesh(b, py::array_t<int>(std::vector<py::ssize_t>{0, 3}));
    return mesh_dist(ma, mb);
  });
  m.def("_mesh_volume", [](py::array_t<double> v, py::array_t<int> t) { return mesh_volume(np_to_mesh(v, t)); });
  // multimerge_ch on parts [(v, t), ...] with their hulls (as process() builds
  // them) and the engine as it stands: the merged hulls.
  m.def("_multimerge", [](py::list parts, double current_concavity, double threshold) {
    MeshList ps, hs;
    for (auto item : parts) {
      auto tup = item.cast<py::tuple>();
      ps.push_back(np_to_mesh(tup[0].cast<py::array_t<double>>(), tup[1].cast<py::array_t<int>>()));
    }
    for (const auto& p : ps) hs.push_back(convex_hull(p.vertices, true));
    multimerge_ch(ps, hs, current_concavity, threshold);
    py::list out;
    for (const auto& h : hs) out.append(mesh_dict(h));
    return out;
  });
  m.def(
      "_separate_disjoint",
      [](py::array_t<double> v, py::array_t<int> t, py::object is_new, py::object edges) {
        Mesh mm = np_to_mesh(v, t);
        if (!is_new.is_none()) {
          auto a = py::array_t<uint8_t, py::array::c_style | py::array::forcecast>(is_new);
          for (py::ssize_t i = 0; i < a.size(); ++i) mm.is_new.push_back(a.data()[i] != 0);
        }
        if (!edges.is_none()) {
          auto a = py::array_t<uint32_t, py::array::c_style | py::array::forcecast>(edges);
          for (py::ssize_t i = 0; i + 1 < a.size(); i += 2) mm.intersecting_edges.push_back({a.data()[i], a.data()[i + 1]});
        }
        MeshList parts{mm};
        separate_disjoint(parts);
        py::list out;
        for (const auto& p : parts) out.append(mesh_dict(p));
        return out;
      },
      py::arg("v"), py::arg("t"), py::arg("is_new") = py::none(), py::arg("edges") = py::none());
  m.def("_visibility", [](py::array_t<double> v, py::array_t<int> t, py::array_t<double> cv, py::array_t<int> ct) {
    Mesh mm = np_to_mesh(v, t), cage = np_to_mesh(cv, ct);
    auto e = gpu::visibility_edges(mm, cage);
    py::array_t<uint32_t> out({(py::ssize_t)e.size(), (py::ssize_t)2});
    for (size_t i = 0; i < e.size(); ++i) {
      out.mutable_at(i, 0) = e[i].first;
      out.mutable_at(i, 1) = e[i].second;
    }
    return out;
  });
}
