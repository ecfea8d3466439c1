#include "core.hpp"

#include <algorithm>
#include <cstring>

namespace visacd {

Vec3 face_normal(const Vec3& p1, const Vec3& p2, const Vec3& p3) {
  Vec3 v = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
  Vec3 w = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
  Vec3 n = cross(v, w);
  double l = std::sqrt(std::pow(n[0], 2) + std::pow(n[1], 2) + std::pow(n[2], 2));
  return {n[0] / l, n[1] / l, n[2] / l};
}

double triangle_area(const Vec3& p0, const Vec3& p1, const Vec3& p2) {
  double a = p1[0] * p0[1] - p2[0] * p0[1] - p0[0] * p1[1] + p2[0] * p1[1] + p0[0] * p2[1] -
             p1[0] * p2[1];
  double b = p1[0] * p0[2] - p2[0] * p0[2] - p0[0] * p1[2] + p2[0] * p1[2] + p0[0] * p2[2] -
             p1[0] * p2[2];
  double c = p1[1] * p0[2] - p2[1] * p0[2] - p0[1] * p1[2] + p2[1] * p1[2] + p0[1] * p2[2] -
             p1[1] * p2[2];
  return 0.5 * std::sqrt(std::pow(a, 2) + std::pow(b, 2) + std::pow(c, 2));
}

Config& config() {
  static Config c;
  return c;
}

CheckerHooks& checker_hooks() {
  static CheckerHooks h;
  return h;
}

std::vector<VisibilityRecord>& recorded_visibility() {
  static std::vector<VisibilityRecord> r;
  return r;
}

std::vector<std::array<double, 5>>& recorded_splits() {
  static std::vector<std::array<double, 5>> r;
  return r;
}

void Mt19937::seed(result_type s) {
  x_[0] = s;
  for (int i = 1; i < kN; ++i) x_[i] = 1812433253u * (x_[i - 1] ^ (x_[i - 1] >> 30)) + (uint32_t)i;
  pos_ = kN;
}

// One pass of the recurrence x_k = x_{k+M} ^ A((x_k & upper) | (x_{k+1} & lower))
// over the state, in runs with fixed index offsets (each run's source words
// are final before it reads them) and trip counts that are multiples of 4 so
// the loops vectorise; then the whole block's outputs are tempered at once.
void Mt19937::twist() {
  auto mix = [](uint32_t a, uint32_t b, uint32_t c) {
    const uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
    return c ^ (y >> 1) ^ ((0u - (y & 1u)) & 0x9908b0dfu);
  };
  static_assert(kN - kM == 227 && kN - 1 - (kN - kM) == 396, "MT19937 run lengths");
  for (int k = 0; k < 224; ++k) x_[k] = mix(x_[k], x_[k + 1], x_[k + kM]);
  for (int k = 224; k < kN - kM; ++k) x_[k] = mix(x_[k], x_[k + 1], x_[k + kM]);
  for (int k = kN - kM; k < kN - 1; ++k) x_[k] = mix(x_[k], x_[k + 1], x_[k + kM - kN]);
  x_[kN - 1] = mix(x_[kN - 1], x_[0], x_[kM - 1]);
  for (int k = 0; k < kN; ++k) out_[k] = temper(x_[k]);
  pos_ = 0;
}

void Mt19937::fill(uint32_t* out, size_t n) {
  while (n > 0) {
    if (pos_ >= kN) twist();
    const size_t take = std::min(n, (size_t)(kN - pos_));
    std::memcpy(out, out_ + pos_, take * sizeof(uint32_t));
    pos_ += (int)take;
    out += take;
    n -= take;
  }
}

namespace {
thread_local Mt19937* tl_engine = nullptr;  // per-thread engine of process_batch workers
}

Mt19937& random_engine() {
  if (tl_engine) return *tl_engine;
  static Mt19937 eng(std::random_device{}());
  return eng;
}

void set_thread_engine(Mt19937* eng) { tl_engine = eng; }

void set_seed(unsigned int seed) { random_engine().seed(seed); }

std::array<double, 6> bbox(const Mesh& m) {
  double xn = kInf, xx = -kInf, yn = kInf, yx = -kInf, zn = kInf, zx = -kInf;
  for (const auto& v : m.vertices) {
    xn = std::min(xn, v[0]);
    xx = std::max(xx, v[0]);
    yn = std::min(yn, v[1]);
    yx = std::max(yx, v[1]);
    zn = std::min(zn, v[2]);
    zx = std::max(zx, v[2]);
  }
  return {xn, xx, yn, yx, zn, zx};
}

std::array<double, 6> normalize(Mesh& m) {
  auto b = bbox(m);
  double len = std::max(std::max(b[1] - b[0], b[3] - b[2]), b[5] - b[4]);
  double mx = (b[1] + b[0]) / 2, my = (b[3] + b[2]) / 2, mz = (b[5] + b[4]) / 2;
  for (auto& v : m.vertices)
    v = {2.0 * (v[0] - mx) / len, 2.0 * (v[1] - my) / len, 2.0 * (v[2] - mz) / len};
  return b;
}

void unnormalize(Mesh& m, const std::array<double, 6>& b) {
  double len = std::max(std::max(b[1] - b[0], b[3] - b[2]), b[5] - b[4]);
  double mx = (b[1] + b[0]) / 2, my = (b[3] + b[2]) / 2, mz = (b[5] + b[4]) / 2;
  for (auto& v : m.vertices)
    v = {v[0] / 2 * len + mx, v[1] / 2 * len + my, v[2] / 2 * len + mz};
}

static double tet_volume(const Vec3& p1, const Vec3& p2, const Vec3& p3) {
  double v321 = p3[0] * p2[1] * p1[2];
  double v231 = p2[0] * p3[1] * p1[2];
  double v312 = p3[0] * p1[1] * p2[2];
  double v132 = p1[0] * p3[1] * p2[2];
  double v213 = p2[0] * p1[1] * p3[2];
  double v123 = p1[0] * p2[1] * p3[2];
  return (1.0 / 6.0) * (-v321 + v231 + v312 - v132 - v213 + v123);
}

double mesh_volume(const Mesh& m) {
  double vol = 0;
  for (const auto& t : m.triangles)
    vol += tet_volume(m.vertices[t[0]], m.vertices[t[1]], m.vertices[t[2]]);
  return vol;
}

}  // namespace visacd
