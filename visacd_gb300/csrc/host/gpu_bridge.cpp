#include "gpu_bridge.hpp"

#include <chrono>
#include <cstring>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "geometry.hpp"
#include "visacd_gpu.h"

namespace visacd {
namespace gpu {

namespace {
void check(int rc, const char* what) {
  if (rc != VISACD_OK)
    throw std::runtime_error(std::string(what) + " failed: " + visacd_last_error());
}
struct BvhHandle {
  visacd_bvh* h = nullptr;
  ~BvhHandle() {
    if (h) visacd_bvh_destroy(h);
  }
};
double now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
}  // namespace

Counters& counters() {
  static thread_local Counters c;
  return c;
}

namespace {
thread_local visacd_ctx* tl_ctx = nullptr;   // a process_batch worker's own context
thread_local visacd_lp* tl_lp = nullptr;     // the proposer on this thread's context
thread_local visacd_ctx* tl_lp_ctx = nullptr;
thread_local std::string tl_lp_path;             // the weights file it was made from
}  // namespace

ThreadContext::ThreadContext(int device, bool blocking_wait) {
  if (visacd_ctx_create(device, nullptr, &ctx_) != VISACD_OK)
    throw std::runtime_error(std::string("cannot create a worker GPU context: ") + visacd_last_error());
  if (blocking_wait) visacd_ctx_set_blocking_wait(ctx_, 1);
  prev_ = tl_ctx;
  tl_ctx = ctx_;
}

ThreadContext::~ThreadContext() {
  if (tl_lp && tl_lp_ctx == ctx_) {
    visacd_lp_destroy(tl_lp);
    tl_lp = nullptr;
    tl_lp_ctx = nullptr;
  }
  tl_ctx = prev_;
  visacd_ctx_destroy(ctx_);
}

int default_device() {
  const char* dev = std::getenv("VISACD_DEVICE");
  return dev ? std::atoi(dev) : 0;
}

visacd_ctx* context() {
  if (tl_ctx) return tl_ctx;
  static std::once_flag once;
  static visacd_ctx* ctx = nullptr;
  static std::string err;
  std::call_once(once, [] {
    if (visacd_ctx_create(default_device(), nullptr, &ctx) != VISACD_OK) {
      err = visacd_last_error();
      ctx = nullptr;
    }
  });
  if (!ctx) throw std::runtime_error("cannot create the GPU context: " + err);
  return ctx;
}

static void to_f32(const std::vector<Vec3>& v, std::vector<float>& out) {
  out.resize(3 * v.size());
  for (size_t i = 0; i < v.size(); ++i)
    for (int k = 0; k < 3; ++k) out[3 * i + k] = (float)v[i][k];
}

std::vector<std::vector<Edge>> visibility_edges_batch(const std::vector<const Mesh*>& parts,
                                                      const std::vector<const Mesh*>& cages) {
  const size_t K = parts.size();
  std::vector<std::vector<Edge>> out(K);
  if (K == 0) return out;
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  std::vector<std::vector<float>> v(K), cv(K);
  std::vector<std::vector<uint8_t>> mask(K);
  std::vector<BvhHandle> sb(K), cb(K);
  std::vector<const float*> pts(K);
  std::vector<int32_t> n(K);
  std::vector<const uint8_t*> masks(K, nullptr);
  std::vector<const visacd_bvh*> sbs(K), cbs(K);
  for (size_t k = 0; k < K; ++k) {
    const Mesh& mesh = *parts[k];
    const Mesh& cage = *cages[k];
    to_f32(mesh.vertices, v[k]);
    to_f32(cage.vertices, cv[k]);
    check(visacd_bvh_build(ctx, v[k].data(), (int32_t)mesh.vertices.size(),
                           reinterpret_cast<const uint32_t*>(mesh.triangles.data()),
                           (int32_t)mesh.triangles.size(), 0, &sb[k].h),
          "visacd_bvh_build(part)");
    check(visacd_bvh_build(ctx, cv[k].data(), (int32_t)cage.vertices.size(),
                           reinterpret_cast<const uint32_t*>(cage.triangles.data()),
                           (int32_t)cage.triangles.size(), 0, &cb[k].h),
          "visacd_bvh_build(cage)");
    if (!mesh.is_new.empty()) {
      mask[k].assign(mesh.vertices.size(), 0);
      for (size_t i = 0; i < mesh.is_new.size() && i < mask[k].size(); ++i) mask[k][i] = mesh.is_new[i] ? 1 : 0;
      masks[k] = mask[k].data();
    }
    pts[k] = v[k].data();
    n[k] = (int32_t)mesh.vertices.size();
    sbs[k] = sb[k].h;
    cbs[k] = cb[k].h;
  }
  std::vector<int64_t> ne(K, 0);
  visacd_vis_stats st;
  check(visacd_visibility_batch(ctx, (int32_t)K, pts.data(), n.data(), masks.data(), sbs.data(), cbs.data(),
                                ne.data(), &st),
        "visacd_visibility_batch");
  int64_t total = 0;
  for (int64_t x : ne) total += x;
  std::vector<uint32_t> flat(2 * (size_t)total);
  check(visacd_visibility_edges(ctx, flat.data(), total), "visacd_visibility_edges");
  int64_t at = 0;
  for (size_t k = 0; k < K; ++k) {
    out[k].resize((size_t)ne[k]);
    for (int64_t e = 0; e < ne[k]; ++e, ++at) out[k][e] = {flat[2 * at], flat[2 * at + 1]};
  }
  if (checker_hooks().record_visibility) {
    for (size_t k = 0; k < K; ++k) {
      VisibilityRecord r{*parts[k], cages[k]->copy_geometry()};
      r.part.intersecting_edges = out[k];
      recorded_visibility().push_back(std::move(r));
    }
  }
  auto& c = counters();
  c.vis_calls++;
  c.vis_pairs += st.pairs_tested;
  c.vis_edges += total;
  c.vis_ms += now_ms() - t0;
  return out;
}

namespace {

// The edge draws of one candidate-plane generation, taken in advance from a
// copy of the process engine: draws[k] is what the reference's
// uniform_int_distribution(0, E - 1) returns at draw k, consumed[k] the engine
// outputs used by draws 0..k (a draw takes more than one when it rejects).
struct DrawPlan {
  std::vector<int32_t> draws;
  std::vector<uint64_t> consumed;
};

struct CountingEngine {
  using result_type = uint32_t;
  Mt19937& eng;
  uint64_t n = 0;
  static constexpr result_type min() { return Mt19937::min(); }
  static constexpr result_type max() { return Mt19937::max(); }
  result_type operator()() {
    ++n;
    return eng();
  }
};

DrawPlan plan_draws(size_t n_edges, int num_planes) {
  DrawPlan plan;
  Mt19937 copy = random_engine();
  CountingEngine ce{copy};
  std::uniform_int_distribution<> dis(0, (int)n_edges - 1);
  const int D = num_planes > 0 ? 5 * num_planes : 0;
  plan.draws.resize(D);
  plan.consumed.resize(D);
  for (int k = 0; k < D; ++k) {
    plan.draws[k] = dis(ce);
    plan.consumed[k] = ce.n;
  }
  return plan;
}

// Moves the process engine past the draws the reference's loop consumed.
void take_draws(const DrawPlan& plan, int32_t draws_used) {
  if (draws_used <= 0) return;
  uint64_t left = plan.consumed[(size_t)draws_used - 1];
  uint32_t sink[256];
  Mt19937& eng = random_engine();
  while (left) {
    const size_t n = left < 256 ? (size_t)left : 256;
    eng.fill(sink, n);
    left -= n;
  }
}

}  // namespace

std::vector<Plane> candidate_planes(const std::vector<Vec3>& vertices, const std::vector<Edge>& edges,
                                    int num_planes) {
  std::vector<Plane> planes;
  if (edges.empty() || num_planes <= 0) return planes;
  visacd_ctx* ctx = context();
  const DrawPlan plan = plan_draws(edges.size(), num_planes);
  std::vector<double> out(4 * (size_t)num_planes);
  int32_t got = 0, used = 0;
  static_assert(sizeof(Edge) == 8, "packed edge pairs");
  check(visacd_candidate_planes(ctx, reinterpret_cast<const double*>(vertices.data()),
                                (int32_t)vertices.size(), reinterpret_cast<const uint32_t*>(edges.data()),
                                (int64_t)edges.size(), plan.draws.data(), (int32_t)plan.draws.size(),
                                num_planes, out.data(), &got, &used),
        "visacd_candidate_planes");
  take_draws(plan, used);
  planes.reserve(got);
  for (int32_t i = 0; i < got; ++i) planes.emplace_back(out[4 * i], out[4 * i + 1], out[4 * i + 2], out[4 * i + 3]);
  return planes;
}

bool split_search(const Mesh& mesh, const std::vector<Plane>& flat_planes, double flat_k, int num_planes,
                  Plane& out) {
  const auto& edges = mesh.intersecting_edges;
  if (edges.empty()) return false;
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  const DrawPlan plan = plan_draws(edges.size(), num_planes);
  std::vector<double> flat(4 * flat_planes.size());
  for (size_t i = 0; i < flat_planes.size(); ++i) {
    flat[4 * i] = flat_planes[i].a;
    flat[4 * i + 1] = flat_planes[i].b;
    flat[4 * i + 2] = flat_planes[i].c;
    flat[4 * i + 3] = flat_planes[i].d;
  }
  double best[4];
  visacd_split_info info{};
  check(visacd_split_search(ctx, reinterpret_cast<const double*>(mesh.vertices.data()),
                            (int32_t)mesh.vertices.size(), reinterpret_cast<const uint32_t*>(edges.data()),
                            (int64_t)edges.size(), plan.draws.data(), (int32_t)plan.draws.size(), num_planes,
                            flat.empty() ? nullptr : flat.data(), (int32_t)flat_planes.size(), flat_k, best,
                            &info),
        "visacd_split_search");
  take_draws(plan, info.draws_used);
  if (checker_hooks().record_visibility)
    recorded_splits().push_back({(double)(info.n_candidates + (int)flat_planes.size()),
                                 (double)mesh.vertices.size(), (double)edges.size(),
                                 (double)info.best_index, info.best_score});
  auto& c = counters();
  c.score_calls++;
  c.plane_edge_pairs += (long long)(info.n_candidates + (int)flat_planes.size()) * (long long)edges.size();
  c.score_ms += now_ms() - t0;
  if (info.best_index < 0) return false;
  out = Plane(best[0], best[1], best[2], best[3]);
  return true;
}

std::vector<Edge> visibility_edges(const Mesh& mesh, const Mesh& cage) {
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  std::vector<float> v, cv;
  to_f32(mesh.vertices, v);
  to_f32(cage.vertices, cv);
  static_assert(sizeof(Tri) == 12 && sizeof(Vec3) == 24, "packed vertex and triangle arrays");
  BvhHandle sb, cb;
  check(visacd_bvh_build(ctx, v.data(), (int32_t)mesh.vertices.size(),
                         reinterpret_cast<const uint32_t*>(mesh.triangles.data()),
                         (int32_t)mesh.triangles.size(), 0, &sb.h),
        "visacd_bvh_build(part)");
  check(visacd_bvh_build(ctx, cv.data(), (int32_t)cage.vertices.size(),
                         reinterpret_cast<const uint32_t*>(cage.triangles.data()),
                         (int32_t)cage.triangles.size(), 0, &cb.h),
        "visacd_bvh_build(cage)");
  std::vector<uint8_t> mask;
  if (!mesh.is_new.empty()) {
    mask.resize(mesh.vertices.size(), 0);
    for (size_t i = 0; i < mesh.is_new.size() && i < mask.size(); ++i) mask[i] = mesh.is_new[i] ? 1 : 0;
  }
  int64_t ne = 0;
  visacd_vis_stats st;
  check(visacd_visibility(ctx, v.data(), (int32_t)mesh.vertices.size(),
                          mask.empty() ? nullptr : mask.data(), 0, sb.h, cb.h, &ne, &st),
        "visacd_visibility");
  std::vector<uint32_t> flat(2 * (size_t)ne);
  check(visacd_visibility_edges(ctx, flat.data(), ne), "visacd_visibility_edges");
  std::vector<Edge> out((size_t)ne);
  for (int64_t k = 0; k < ne; ++k) out[k] = {flat[2 * k], flat[2 * k + 1]};
  auto& c = counters();
  c.vis_calls++;
  c.vis_pairs += st.pairs_tested;
  c.vis_edges += ne;
  c.vis_ms += now_ms() - t0;
  return out;
}

std::vector<double> score_planes(const std::vector<Plane>& planes, const std::vector<Vec3>& pts,
                                 const std::vector<Edge>& edges) {
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  std::vector<float> pl(4 * planes.size()), p;
  for (size_t i = 0; i < planes.size(); ++i) {
    pl[4 * i] = (float)planes[i].a;
    pl[4 * i + 1] = (float)planes[i].b;
    pl[4 * i + 2] = (float)planes[i].c;
    pl[4 * i + 3] = (float)planes[i].d;
  }
  to_f32(pts, p);
  std::vector<uint32_t> e(2 * edges.size());
  for (size_t k = 0; k < edges.size(); ++k) {
    e[2 * k] = edges[k].first;
    e[2 * k + 1] = edges[k].second;
  }
  std::vector<double> scores(planes.size(), 0.0);
  check(visacd_score_planes(ctx, pl.data(), (int32_t)planes.size(), p.data(), (int32_t)pts.size(),
                            e.data(), (int64_t)edges.size(), 0, scores.data(), nullptr),
        "visacd_score_planes");
  auto& c = counters();
  c.score_calls++;
  c.plane_edge_pairs += (long long)planes.size() * (long long)edges.size();
  c.score_ms += now_ms() - t0;
  return scores;
}

double face_hausdorff(const Mesh& A, const std::vector<Vec3>& XA, const std::vector<int>& idA,
                      const Mesh& B, const std::vector<Vec3>& XB, const std::vector<int>& idB,
                      double floor) {
  visacd_ctx* ctx = context();
  double out = 0;
  check(visacd_face_hausdorff_floor(ctx, reinterpret_cast<const double*>(A.vertices.data()), (int32_t)A.vertices.size(),
                              reinterpret_cast<const int32_t*>(A.triangles.data()), (int32_t)A.triangles.size(),
                              reinterpret_cast<const double*>(XA.data()), idA.data(), (int32_t)XA.size(),
                              reinterpret_cast<const double*>(B.vertices.data()), (int32_t)B.vertices.size(),
                              reinterpret_cast<const int32_t*>(B.triangles.data()), (int32_t)B.triangles.size(),
                              reinterpret_cast<const double*>(XB.data()), idB.data(), (int32_t)XB.size(), floor,
                              &out),
        "visacd_face_hausdorff_floor");
  return out;
}

std::vector<double> face_hausdorff_batch(const std::vector<const Mesh*>& a, const std::vector<const Mesh*>& b,
                                         const std::vector<const HbSamples*>& s, const std::vector<double>& lower,
                                         double floor, bool independent) {
  const size_t J = a.size();
  std::vector<double> out(J, 0.0);
  if (J == 0) return out;
  visacd_ctx* ctx = context();
  // Concatenated surfaces: mesh / set 2j = a[j], 2j + 1 = b[j].
  thread_local std::vector<double> V, X;
  thread_local std::vector<int32_t> T, I;
  std::vector<int64_t> voff(2 * J + 1, 0), toff(2 * J + 1, 0), soff(2 * J + 1, 0);
  for (size_t j = 0; j < J; ++j) {
    const Mesh* m[2] = {a[j], b[j]};
    const size_t ns[2] = {s[j]->s1.size(), s[j]->s2.size()};
    for (int k = 0; k < 2; ++k) {
      voff[2 * j + k + 1] = voff[2 * j + k] + (int64_t)m[k]->vertices.size();
      toff[2 * j + k + 1] = toff[2 * j + k] + (int64_t)m[k]->triangles.size();
      soff[2 * j + k + 1] = soff[2 * j + k] + (int64_t)ns[k];
    }
  }
  V.resize(3 * (size_t)voff[2 * J]);
  T.resize(3 * (size_t)toff[2 * J]);
  X.resize(3 * (size_t)soff[2 * J]);
  I.resize((size_t)soff[2 * J]);
  for (size_t j = 0; j < J; ++j) {
    const Mesh* m[2] = {a[j], b[j]};
    const std::vector<Vec3>* xs[2] = {&s[j]->s1, &s[j]->s2};
    const std::vector<int>* is[2] = {&s[j]->i1, &s[j]->i2};
    for (int k = 0; k < 2; ++k) {
      const size_t q = 2 * j + k;
      std::memcpy(V.data() + 3 * voff[q], m[k]->vertices.data(), m[k]->vertices.size() * 24);
      std::memcpy(T.data() + 3 * toff[q], m[k]->triangles.data(), m[k]->triangles.size() * 12);
      std::memcpy(X.data() + 3 * soff[q], xs[k]->data(), xs[k]->size() * 24);
      std::memcpy(I.data() + soff[q], is[k]->data(), is[k]->size() * 4);
    }
  }
  check(visacd_face_hausdorff_batch(ctx, (int32_t)J, V.data(), voff.data(), T.data(), toff.data(), X.data(),
                                    I.data(), soff.data(), lower.empty() ? nullptr : lower.data(), floor,
                                    independent ? 1 : 0, out.data()),
        "visacd_face_hausdorff_batch");
  return out;
}

MeshList clip(const Mesh& mesh, const Plane& plane, std::vector<int>& pos_map,
              std::vector<int>& neg_map) {
  visacd_ctx* ctx = context();
  const int nv = (int)mesh.vertices.size(), nt = (int)mesh.triangles.size();
  const double pl[4] = {plane.a, plane.b, plane.c, plane.d};
  visacd_clip_result r;
  check(visacd_clip(ctx, reinterpret_cast<const double*>(mesh.vertices.data()), nv,
                    reinterpret_cast<const int32_t*>(mesh.triangles.data()), nt, pl, &r),
        "visacd_clip");
  std::vector<Tri> pt(r.n_pos), ng(r.n_neg);
  pos_map.assign(nv, 0);
  neg_map.assign(nv, 0);
  std::vector<Vec3> border(r.n_border);
  std::vector<int32_t> be(2 * (size_t)r.n_border_edges);
  check(visacd_clip_fetch(ctx, reinterpret_cast<int32_t*>(pt.data()),
                          reinterpret_cast<int32_t*>(ng.data()), pos_map.data(), neg_map.data(),
                          reinterpret_cast<double*>(border.data()), be.data()),
        "visacd_clip_fetch");
  std::vector<std::pair<int, int>> bedges(r.n_border_edges);
  for (int k = 0; k < r.n_border_edges; ++k) bedges[k] = {be[2 * k], be[2 * k + 1]};
  return assemble_clip(mesh, plane, pt, ng, pos_map, neg_map, border, bedges);
}

void sdf_remesh(Mesh& m, double scale, double level) {
  visacd_ctx* ctx = context();
  std::vector<double> v(3 * m.vertices.size());
  for (size_t i = 0; i < m.vertices.size(); ++i)
    for (int k = 0; k < 3; ++k) v[3 * i + k] = m.vertices[i][k];
  int32_t nv = 0, nt = 0;
  check(visacd_sdf_remesh(ctx, v.data(), (int32_t)m.vertices.size(),
                          reinterpret_cast<const int32_t*>(m.triangles.data()), (int32_t)m.triangles.size(),
                          scale, level, &nv, &nt),
        "visacd_sdf_remesh");
  std::vector<Vec3> ov(nv);
  std::vector<Tri> ot(nt);
  check(visacd_sdf_fetch(ctx, reinterpret_cast<double*>(ov.data()), reinterpret_cast<int32_t*>(ot.data())),
        "visacd_sdf_fetch");
  m.clear();
  m.is_new.clear();
  m.intersecting_edges.clear();
  m.vertices = std::move(ov);
  m.triangles = std::move(ot);
}

MeshList convex_hulls(const std::vector<const std::vector<Vec3>*>& sets, bool fix_normals) {
  MeshList out(sets.size());
  if (sets.empty()) return out;
  visacd_ctx* ctx = context();
  std::vector<int64_t> off(sets.size() + 1, 0);
  for (size_t k = 0; k < sets.size(); ++k) off[k + 1] = off[k] + (int64_t)sets[k]->size();
  std::vector<double> v;
  v.reserve(3 * (size_t)off.back());
  for (const auto* s : sets)
    for (const auto& p : *s) v.insert(v.end(), p.begin(), p.end());
  std::vector<int32_t> tris(6 * (size_t)off.back()), counts(sets.size());
  check(visacd_convex_hulls(ctx, v.data(), off.data(), (int32_t)sets.size(), fix_normals ? 1 : 0, tris.data(),
                            counts.data()),
        "visacd_convex_hulls");
  for (size_t k = 0; k < sets.size(); ++k) {
    out[k].vertices = *sets[k];
    const int32_t* t = tris.data() + 6 * off[k];
    out[k].triangles.resize(counts[k]);
    for (int32_t i = 0; i < counts[k]; ++i) out[k].triangles[i] = {t[3 * i], t[3 * i + 1], t[3 * i + 2]};
  }
  return out;
}

std::vector<double> hull_distances(const MeshList& hulls, const std::vector<std::pair<int, int>>& pairs,
                                   double cutoff) {
  std::vector<double> out(pairs.size());
  if (pairs.empty()) return out;
  visacd_ctx* ctx = context();
  std::vector<int64_t> off(hulls.size() + 1, 0);
  for (size_t h = 0; h < hulls.size(); ++h) off[h + 1] = off[h] + (int64_t)hulls[h].vertices.size();
  std::vector<double> v;
  v.reserve(3 * (size_t)off.back());
  for (const auto& h : hulls)
    for (const auto& p : h.vertices) v.insert(v.end(), p.begin(), p.end());
  std::vector<int32_t> pr(2 * pairs.size());
  for (size_t k = 0; k < pairs.size(); ++k) {
    pr[2 * k] = pairs[k].first;
    pr[2 * k + 1] = pairs[k].second;
  }
  check(visacd_hull_distances(ctx, v.data(), off.data(), (int32_t)hulls.size(), pr.data(), (int64_t)pairs.size(),
                              cutoff, out.data()),
        "visacd_hull_distances");
  return out;
}

namespace {
// Proposer parameters by file path, read once per path.
std::shared_ptr<const std::vector<float>> proposer_params(const std::string& path) {
  static std::mutex mu;
  static std::string loaded_path;
  static std::shared_ptr<const std::vector<float>> params;
  std::lock_guard<std::mutex> lock(mu);
  if (path.empty())
    throw std::runtime_error("plane_proposer is 'learned' but config.proposer_weights is empty");
  if (path != loaded_path) {
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open proposer weights " + path);
    const int n = visacd_lp_param_count();
    std::vector<float> p(n);
    const size_t got = std::fread(p.data(), sizeof(float), n, f);
    const bool extra = std::fgetc(f) != EOF;
    std::fclose(f);
    if (got != (size_t)n || extra)
      throw std::runtime_error("proposer weights " + path + " must hold exactly " + std::to_string(n) +
                               " float32 values");
    params = std::make_shared<const std::vector<float>>(std::move(p));
    loaded_path = path;
  }
  return params;
}
}  // namespace

namespace {
// This thread's proposer on its context, made from config().proposer_weights.
visacd_lp* proposer(visacd_ctx* ctx) {
  if (!tl_lp || tl_lp_ctx != ctx || tl_lp_path != config().proposer_weights) {
    if (tl_lp) visacd_lp_destroy(tl_lp);
    tl_lp = nullptr;
    const auto p = proposer_params(config().proposer_weights);
    check(visacd_lp_create(ctx, p->data(), 0, &tl_lp), "visacd_lp_create");
    tl_lp_ctx = ctx;
    tl_lp_path = config().proposer_weights;
  }
  return tl_lp;
}

// The part's frame for the proposer: bounding-box centre (float) and half of
// the longest extent (1 for a point).
void part_frame(const Mesh& mesh, float center[3], double& half) {
  auto b = bbox(mesh);
  center[0] = (float)(0.5 * (b[0] + b[1]));
  center[1] = (float)(0.5 * (b[2] + b[3]));
  center[2] = (float)(0.5 * (b[4] + b[5]));
  half = 0.5 * std::max(b[1] - b[0], std::max(b[3] - b[2], b[5] - b[4]));
  if (!(half > 0)) half = 1.0;
}
}  // namespace

std::vector<Plane> propose_planes(const Mesh& mesh) {
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  visacd_lp* lp = proposer(ctx);
  float center[3];
  double half;
  part_frame(mesh, center, half);
  std::vector<float> v;
  to_f32(mesh.vertices, v);
  std::vector<uint32_t> e(2 * mesh.intersecting_edges.size());
  for (size_t k = 0; k < mesh.intersecting_edges.size(); ++k) {
    e[2 * k] = mesh.intersecting_edges[k].first;
    e[2 * k + 1] = mesh.intersecting_edges[k].second;
  }
  double out[VISACD_LP_PLANES * 4];
  check(visacd_lp_propose(lp, v.data(), (int32_t)mesh.vertices.size(), e.data(),
                          (int64_t)mesh.intersecting_edges.size(), center, (float)half, out),
        "visacd_lp_propose");
  std::vector<Plane> planes;
  for (int q = 0; q < VISACD_LP_PLANES; ++q)
    planes.emplace_back(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
  auto& c = counters();
  c.lp_calls++;
  c.lp_ms += now_ms() - t0;
  return planes;
}

bool learned_split_search(const Mesh& mesh, const std::vector<Plane>& flat_planes, double flat_k, Plane& out,
                          bool& fallback) {
  const auto& edges = mesh.intersecting_edges;
  fallback = false;
  if (edges.empty()) return false;
  double t0 = now_ms();
  visacd_ctx* ctx = context();
  visacd_lp* lp = proposer(ctx);
  float center[3];
  double half;
  part_frame(mesh, center, half);
  const int probe = config().proposer_probe_planes;
  const DrawPlan plan = plan_draws(edges.size(), probe);
  std::vector<double> flat(4 * flat_planes.size());
  for (size_t i = 0; i < flat_planes.size(); ++i) {
    flat[4 * i] = flat_planes[i].a;
    flat[4 * i + 1] = flat_planes[i].b;
    flat[4 * i + 2] = flat_planes[i].c;
    flat[4 * i + 3] = flat_planes[i].d;
  }
  double best[4];
  visacd_learned_split_info info{};
  check(visacd_learned_split_search(lp, reinterpret_cast<const double*>(mesh.vertices.data()),
                                    (int32_t)mesh.vertices.size(), reinterpret_cast<const uint32_t*>(edges.data()),
                                    (int64_t)edges.size(), center, (float)half, half, config().proposer_refine,
                                    plan.draws.data(), (int32_t)plan.draws.size(), probe,
                                    flat.empty() ? nullptr : flat.data(), (int32_t)flat_planes.size(), flat_k,
                                    config().proposer_tolerance, best, &info),
        "visacd_learned_split_search");
  take_draws(plan, info.draws_used);
  auto& c = counters();
  c.lp_calls++;
  c.score_calls++;
  c.plane_edge_pairs +=
      (long long)(VISACD_LP_PLANES + info.n_refined + info.n_probe + (int)flat_planes.size()) * (long long)edges.size();
  c.lp_ms += now_ms() - t0;
  if (info.fallback) {
    fallback = true;
    return false;
  }
  if (info.best_index < 0) return false;
  out = Plane(best[0], best[1], best[2], best[3]);
  return true;
}

}  // namespace gpu
}  // namespace visacd

namespace visacd {

// SDF remesh dispatch (lib/src/preprocess.cpp:18-67): the GPU kernels, or the
// host restatement they equal (test hook checker_hooks().host_remesh).
void manifold_preprocess(Mesh& m, double scale, double level) {
  if (!checker_hooks().host_remesh)
    gpu::sdf_remesh(m, scale, level);
  else
    manifold_preprocess_host(m, scale, level);
}

}  // namespace visacd
