// ORACLE -- test infrastructure only.
//
// A CPU restatement of feriphys's spring-mass-damper (cloth) step, used as the
// oracle of the CUDA path in tests/, in __graft_entry__.smoke() and as the
// timed CPU baseline in bench.py.  Nothing in the shipped library links it.
//
// The reference is a Rust crate that cannot be built here (no cargo/rustc),
// so this file restates, in C++, the algorithm of:
//   src/simulation/springy/springy_mesh.rs   (Strut 57-91, Face 110-173,
//        Point 176-256, SpringyMesh::new 267-401, add_strut 403-413,
//        add_pin 415-417, update_points 423-497, get_vertices 500-513,
//        accumulate_forces 515-525, apply_external_point_forces 527-531,
//        apply_strut_forces 533-551, apply_face_forces 629-654,
//        clear_forces 656-660)
//   src/simulation/springy/cloth.rs          (Cloth::new 20-113)
//   src/simulation/springy/simulation.rs     (Simulation::step 27-45)
//   src/simulation/springy/config.rs         (Config + defaults 9-33)
//   src/simulation/state.rs                  (State 41-113: euler 75-83, rk4 86-106)
//   src/simulation/collidable_mesh.rs        (Face 40-47, CollidableMesh::new 57-97,
//        get_collided_face_from_list 107-169)
//   src/utils.rs                             (vec_add 5-14, scale 16-21)
//   src/simulation/consts.rs                 (EPSILON = 1e-4, line 2)
// The vector arithmetic follows cgmath 0.18.0 (Cargo.lock), a dependency that
// is not vendored with the reference; its documented semantics are restated:
//   dot = (x*x' + y*y') + z*z'; magnitude = sqrt(dot(v, v));
//   normalize(v) = v * (1 / magnitude(v)); cross = the usual component formula;
//   Vector3::angle(a, b) = atan2(|a x b|, a . b).
// Every expression keeps the reference's evaluation order, and this file must
// be compiled with -ffp-contract=off (Rust never fuses a*b+c).
//
// Parity pins: tests/test_oracle_golden.py checks this restatement against the
// assertions of the reference's own unit tests (springy_mesh.rs:721-883,
// state.rs:166-280, collidable_mesh.rs:219-269, utils.rs:42-54) and against
// hand-derived known answers for the force, aerodynamic and collision terms,
// which no reference test pins.
//
// The template parameter S is the arithmetic type.  S = float is the faithful
// restatement; S = double is the same algorithm on widened inputs, used only to
// check the FP64 rerun of the GPU step.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- vectors ---
template <class S>
struct V3 {
  S x, y, z;
};
template <class S> static inline V3<S> vadd(V3<S> a, V3<S> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S> static inline V3<S> vsub(V3<S> a, V3<S> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S> static inline V3<S> smul(S s, V3<S> v) { return {s * v.x, s * v.y, s * v.z}; }
template <class S> static inline V3<S> vmuls(V3<S> v, S s) { return {v.x * s, v.y * s, v.z * s}; }
template <class S> static inline V3<S> vdivs(V3<S> v, S s) { return {v.x / s, v.y / s, v.z / s}; }
template <class S> static inline S dot(V3<S> a, V3<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S> static inline V3<S> cross(V3<S> a, V3<S> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float sq_root(float v) { return std::sqrt(v); }
static inline double sq_root(double v) { return std::sqrt(v); }
static inline float arctan2(float y, float x) { return std::atan2(y, x); }
static inline double arctan2(double y, double x) { return std::atan2(y, x); }
template <class S> static inline S magnitude(V3<S> v) { return sq_root(dot(v, v)); }
template <class S> static inline V3<S> normalize(V3<S> v) { return vmuls(v, S(1) / magnitude(v)); }
template <class S> static inline S angle(V3<S> a, V3<S> b) { return arctan2(magnitude(cross(a, b)), dot(a, b)); }
template <class S> static inline bool is_zero(V3<S> v) { return v.x == S(0) && v.y == S(0) && v.z == S(0); }
template <class S> static inline bool sign_positive(S v) { return !std::signbit(v); }
template <class S> static inline V3<S> zero3() { return {S(0), S(0), S(0)}; }

// std::f32::consts::PI and consts::EPSILON as f32; the f64 variant widens them.
static const float PI_F32 = 3.14159265358979323846f;
static const float EPSILON_F32 = 0.0001f;

// Rust's Duration::from_secs_f32(x).as_secs_f32() (Rust >= 1.63): x is rounded
// to whole nanoseconds (nearest, ties to even) and converted back as
// secs as f32 + nanos as f32 / 1e9.  `x` must be finite and >= 0.
float duration_roundtrip(float x) {
  uint32_t bits;
  std::memcpy(&bits, &x, 4);
  const int biased = int((bits >> 23) & 0xffu);
  const uint32_t frac = bits & 0x7fffffu;
  if (biased == 0 && frac == 0) return 0.0f;
  uint64_t m;
  int e2;  // x = m * 2^e2
  if (biased == 0) { m = frac; e2 = -149; } else { m = frac | 0x800000u; e2 = biased - 150; }
  unsigned __int128 p = (unsigned __int128)m * 1000000000u;  // x * 1e9 = p * 2^e2
  unsigned __int128 total;
  if (e2 >= 0) {
    total = p << e2;  // callers keep x far below 2^64 s
  } else {
    const int s = -e2;
    if (s >= 120) return 0.0f;
    const unsigned __int128 one = 1;
    unsigned __int128 q = p >> s;
    const unsigned __int128 rem = p & ((one << s) - 1);
    const unsigned __int128 half = one << (s - 1);
    if (rem > half || (rem == half && (q & 1))) q += 1;
    total = q;
  }
  const uint64_t secs = uint64_t(total / 1000000000u);
  const uint32_t nanos = uint32_t(total % 1000000000u);
  return float(secs) + float(nanos) / 1000000000.0f;
}

// ------------------------------------------------------------------ State ---
// state.rs:10-16 (Stateful) and 41-113 (State).
template <class S>
static std::vector<S> vec_add(const std::vector<S>& a, const std::vector<S>& b) {  // utils.rs:5-14
  if (a.size() != b.size()) throw std::runtime_error("Cannot multiply vectors of different lengths!");
  std::vector<S> out(a.size());
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i] + b[i];
  return out;
}
template <class S>
static std::vector<S> scale(const std::vector<S>& v, S s) {  // utils.rs:16-21
  std::vector<S> out(v.size());
  for (size_t i = 0; i < v.size(); ++i) out[i] = v[i] * s;
  return out;
}

template <class S, class E>
struct State {
  std::vector<E> elements;

  static State from_state_vector(const std::vector<S>& sv) {  // state.rs:46-54
    const size_t n = E::num_state_elements();
    State st;
    st.elements.reserve(sv.size() / n + 1);
    for (size_t i = 0; i < sv.size(); i += n) {
      const size_t end = std::min(sv.size(), i + n);
      st.elements.push_back(E::from_state_vector(std::vector<S>(sv.begin() + i, sv.begin() + end)));
    }
    return st;
  }
  std::vector<S> derivative() const {  // state.rs:56-62
    std::vector<S> out;
    for (const E& e : elements) {
      std::vector<S> d = e.derivative();
      out.insert(out.end(), d.begin(), d.end());
    }
    return out;
  }
  std::vector<S> as_vector() const {  // state.rs:64-70
    std::vector<S> out;
    for (const E& e : elements) {
      std::vector<S> d = e.as_state();
      out.insert(out.end(), d.begin(), d.end());
    }
    return out;
  }
  State euler_step(S h) const {  // state.rs:75-83
    std::vector<S> delta = derivative();
    for (S& x : delta) x = x * h;
    return from_state_vector(vec_add(as_vector(), delta));
  }
  State rk4_step(S h) const {  // state.rs:86-106
    const std::vector<S> k1 = derivative();
    const std::vector<S> half_k1 = scale(k1, h * S(0.5));
    const std::vector<S> k2 = from_state_vector(vec_add(as_vector(), half_k1)).derivative();
    const std::vector<S> half_k2 = scale(k2, h * S(0.5));
    const std::vector<S> k3 = from_state_vector(vec_add(as_vector(), half_k2)).derivative();
    const std::vector<S> k3d = scale(k3, h);
    const std::vector<S> k4 = from_state_vector(vec_add(as_vector(), k3d)).derivative();
    std::vector<S> delta(k1.size());
    for (size_t i = 0; i < k1.size(); ++i)
      delta[i] = h / S(6) * k1[i] + h / S(3) * k2[i] + h / S(3) * k3[i] + h / S(6) * k4[i];
    return from_state_vector(vec_add(as_vector(), delta));
  }
};

// ------------------------------------------------------------------ Point ---
// springy_mesh.rs:176-256.
template <class S>
struct Point {
  S mass;
  V3<S> position, velocity, accumulated_force;

  static size_t num_state_elements() { return 10; }
  static Point from_state_vector(const std::vector<S>& d) {
    if (d.size() != 10) throw std::runtime_error("State Vector incorrect size!");
    return Point{d[0], {d[1], d[2], d[3]}, {d[4], d[5], d[6]}, {d[7], d[8], d[9]}};
  }
  std::vector<S> derivative() const {
    return {S(0), velocity.x, velocity.y, velocity.z,
            accumulated_force.x / mass, accumulated_force.y / mass, accumulated_force.z / mass,
            S(0), S(0), S(0)};
  }
  std::vector<S> as_state() const {
    return {mass, position.x, position.y, position.z, velocity.x, velocity.y, velocity.z,
            accumulated_force.x, accumulated_force.y, accumulated_force.z};
  }
};

// ----------------------------------------------------------- Collidables ---
// collidable_mesh.rs:40-47 (Face), 57-97 (new), 107-169 (first-hit search).
template <class S>
struct CFace {
  V3<S> v0, v1, v2;
  V3<S> normal() const { return normalize(cross(vsub(v1, v0), vsub(v2, v0))); }
  S distance_from_plane(V3<S> p) const { return dot(vsub(p, v0), normal()); }
};

template <class S>
struct CollidableMesh {
  std::vector<V3<S>> vertices;
  std::vector<std::pair<V3<S>, V3<S>>> edges;
  std::vector<CFace<S>> faces;

  static CollidableMesh make(const std::vector<V3<S>>& pos, const std::vector<uint64_t>& idx) {
    CollidableMesh m;
    m.vertices = pos;
    // BTreeSet<BTreeSet<&usize>>: unique index pairs in lexicographic order.
    std::set<std::pair<uint64_t, uint64_t>> es;
    const size_t nt = idx.size() / 3;
    for (size_t t = 0; t < nt; ++t) {
      const uint64_t a = idx[3 * t], b = idx[3 * t + 1], c = idx[3 * t + 2];
      if (a >= pos.size() || b >= pos.size() || c >= pos.size())
        throw std::out_of_range("collidable mesh index out of range");
      if (a == b || b == c || c == a)
        throw std::invalid_argument("collidable mesh triangle repeats a vertex");
      es.insert({std::min(a, b), std::max(a, b)});
      es.insert({std::min(b, c), std::max(b, c)});
      es.insert({std::min(c, a), std::max(c, a)});
    }
    for (const auto& e : es) m.edges.push_back({pos[e.first], pos[e.second]});
    for (size_t t = 0; t < nt; ++t)
      m.faces.push_back(CFace<S>{pos[idx[3 * t]], pos[idx[3 * t + 1]], pos[idx[3 * t + 2]]});
    return m;
  }
};

// Returns the index (into `faces`) of the first face the segment crosses, or -1.
// `dt` is Duration::as_secs_f32() of the step's Duration, widened for S=double.
template <class S>
static long collided_face(const std::vector<const CFace<S>*>& faces, V3<S> old_position,
                          V3<S> new_position, S dt) {
  for (size_t i = 0; i < faces.size(); ++i) {
    const CFace<S>& face = *faces[i];
    const V3<S> old_velocity = vdivs(vsub(new_position, old_position), dt);
    const S old_d = face.distance_from_plane(old_position);
    const S new_d = face.distance_from_plane(new_position);
    const bool crossed = sign_positive(old_d) != sign_positive(new_d);
    if (!crossed) continue;
    const S fraction = old_d / (old_d - new_d);
    const V3<S> cp = vadd(old_position, smul(dt * fraction, old_velocity));
    const V3<S> n = face.normal();
    V3<S> a, b, c, p;
    if (n.x >= n.y && n.x >= n.z) {
      a = {S(0), face.v0.y, face.v0.z}; b = {S(0), face.v1.y, face.v1.z};
      c = {S(0), face.v2.y, face.v2.z}; p = {S(0), cp.y, cp.z};
    } else if (n.y >= n.x && n.y >= n.z) {
      a = {face.v0.x, S(0), face.v0.z}; b = {face.v1.x, S(0), face.v1.z};
      c = {face.v2.x, S(0), face.v2.z}; p = {cp.x, S(0), cp.z};
    } else {
      a = {face.v0.x, face.v0.y, S(0)}; b = {face.v1.x, face.v1.y, S(0)};
      c = {face.v2.x, face.v2.y, S(0)}; p = {cp.x, cp.y, S(0)};
    }
    const V3<S> c0 = cross(vsub(b, a), vsub(p, a));
    const V3<S> c1 = cross(vsub(c, b), vsub(p, b));
    const V3<S> c2 = cross(vsub(a, c), vsub(p, c));
    const bool o0 = sign_positive(dot(c0, face.normal()));
    const bool o1 = sign_positive(dot(c1, face.normal()));
    const bool o2 = sign_positive(dot(c2, face.normal()));
    if (o0 == o1 && o1 == o2) return long(i);
  }
  return -1;
}

// ----------------------------------------------------------------- Config ---
// config.rs:9-33.  integration: 0 = Euler, 1 = Rk4 (state.rs:4-8).
template <class S>
struct Config {
  int integration;
  float dt;  // seconds as f32 (the reference keeps dt in f32)
  V3<S> gravity, wind;
  S lift_coefficient, drag_coefficient, coefficient_of_restitution, coefficient_of_friction;
};

// ------------------------------------------------------------ SpringyMesh ---
template <class S>
struct Strut {  // springy_mesh.rs:57-91
  S stiffness, damping, length;
  uint64_t a, b;
  long f0, f1;  // adjacent faces, -1 = None
};
struct MeshFace {  // springy_mesh.rs:110-115
  uint64_t s0, s1, s2;
  uint64_t v0, v1, v2;
};

struct PairHash {
  size_t operator()(const std::pair<uint64_t, uint64_t>& k) const {
    return std::hash<uint64_t>()(k.first * 0x9E3779B97F4A7C15ull ^ (k.second + 0x632BE59BD9B4E019ull));
  }
};
using KeyMap = std::unordered_map<std::pair<uint64_t, uint64_t>, std::pair<float, float>, PairHash>;

static inline std::pair<uint64_t, uint64_t> strut_key(uint64_t a, uint64_t b) {  // StrutKey::new 101-106
  return a <= b ? std::make_pair(a, b) : std::make_pair(b, a);
}

template <class S>
struct SpringyMesh {
  std::vector<Strut<S>> struts;
  std::vector<MeshFace> faces;
  std::vector<Point<S>> points;
  std::vector<uint64_t> pinned_points;

  // Strut::new 74-90: stiffness = NOMINAL_STRUT_LENGTH / length * nominal.
  static Strut<S> make_strut(float k, float c, float length, uint64_t a, uint64_t b) {
    return Strut<S>{S(1.0f / length * k), S(1.0f / length * c), S(length), a, b, -1, -1};
  }

  // SpringyMesh::new 267-401 (f32 construction; torsional springs are not
  // built: the reference's Cloth passes None and the force is disabled, 518-519).
  static SpringyMesh make(const std::vector<V3<float>>& pos, const std::vector<uint64_t>& idx, float mass,
                          float default_stiffness, float default_damping, const KeyMap* overrides) {
    SpringyMesh m;
    const float mass_per_vert = mass / float(pos.size());
    m.points.reserve(pos.size());
    for (const auto& p : pos)
      m.points.push_back(Point<S>{S(mass_per_vert), {S(p.x), S(p.y), S(p.z)}, zero3<S>(), zero3<S>()});
    std::unordered_map<std::pair<uint64_t, uint64_t>, uint64_t, PairHash> index;
    index.reserve(idx.size());
    const size_t nt = idx.size() / 3;
    for (size_t i = 0; i < 3 * nt; ++i)
      if (idx[i] >= pos.size()) throw std::out_of_range("vertex index out of range");
    auto add = [&](uint64_t i1, uint64_t i2) {
      const auto key = strut_key(i1, i2);
      if (index.find(key) != index.end()) return;
      index.emplace(key, m.struts.size());
      float k = default_stiffness, c = default_damping;
      if (overrides) {
        auto it = overrides->find(key);
        if (it != overrides->end()) { k = it->second.first; c = it->second.second; }
      }
      const V3<float> d = vsub(pos[key.first], pos[key.second]);
      m.struts.push_back(make_strut(k, c, magnitude(d), key.first, key.second));
    };
    for (size_t t = 0; t < nt; ++t) {
      const uint64_t v0 = idx[3 * t], v1 = idx[3 * t + 1], v2 = idx[3 * t + 2];
      add(v0, v1);
      add(v1, v2);
      add(v2, v0);
    }
    for (size_t t = 0; t < nt; ++t) {
      const uint64_t v0 = idx[3 * t], v1 = idx[3 * t + 1], v2 = idx[3 * t + 2];
      const uint64_t s0 = index.at(strut_key(v0, v1));
      const uint64_t s1 = index.at(strut_key(v1, v2));
      const uint64_t s2 = index.at(strut_key(v2, v0));
      const long face_index = long(m.faces.size());
      m.faces.push_back(MeshFace{s0, s1, s2, v0, v1, v2});
      for (uint64_t s : {s0, s1, s2}) {
        Strut<S>& st = m.struts[s];
        if (st.f0 < 0) st.f0 = face_index;
        else if (st.f1 < 0) st.f1 = face_index;
        else throw std::invalid_argument("A strut shouldn't have more than two adjacent faces!");
      }
    }
    return m;
  }

  // add_strut 403-413: the vertex order is kept as given.
  void add_strut(uint64_t a, uint64_t b, float k, float c) {
    if (a >= points.size() || b >= points.size()) throw std::out_of_range("strut vertex out of range");
    const V3<float> pa{float(points[a].position.x), float(points[a].position.y), float(points[a].position.z)};
    const V3<float> pb{float(points[b].position.x), float(points[b].position.y), float(points[b].position.z)};
    struts.push_back(make_strut(k, c, magnitude(vsub(pa, pb)), a, b));
  }
  void add_pin(uint64_t i) {  // 415-417
    if (i >= points.size()) throw std::out_of_range("pin index out of range");
    pinned_points.push_back(i);
  }

  V3<S> face_normal(const MeshFace& f) const {  // 118-124
    const V3<S> x0 = points[f.v0].position, x1 = points[f.v1].position, x2 = points[f.v2].position;
    return normalize(cross(vsub(x1, x0), vsub(x2, x0)));
  }
  S face_area(const MeshFace& f) const {  // 126-131
    const V3<S> x0 = points[f.v0].position, x1 = points[f.v1].position, x2 = points[f.v2].position;
    return magnitude(cross(vsub(x1, x0), vsub(x2, x0))) / S(2);
  }
  S vertex_angle(uint64_t i0, uint64_t i1, uint64_t i2) const {  // 163-172
    return angle(vsub(points[i2].position, points[i0].position), vsub(points[i1].position, points[i0].position));
  }
  S vertex_angle_k(const MeshFace& f, int k) const {  // 134-161
    if (k == 0) return vertex_angle(f.v0, f.v1, f.v2);
    if (k == 1) return vertex_angle(f.v1, f.v2, f.v0);
    return vertex_angle(f.v2, f.v0, f.v1);
  }

  void apply_external_point_forces(const Config<S>& cfg) {  // 527-531, 194-196
    for (auto& p : points) p.accumulated_force = vadd(p.accumulated_force, cfg.gravity);
  }
  void apply_strut_forces() {  // 533-551
    for (const auto& s : struts) {
      const V3<S> p0 = points[s.a].position, p1 = points[s.b].position;
      const V3<S> u = normalize(vsub(p1, p0));
      const V3<S> sf = smul(s.stiffness * (magnitude(vsub(p1, p0)) - s.length), u);
      points[s.a].accumulated_force = vadd(points[s.a].accumulated_force, sf);
      points[s.b].accumulated_force = vadd(points[s.b].accumulated_force, smul(S(-1), sf));
      const V3<S> v0 = points[s.a].velocity, v1 = points[s.b].velocity;
      const V3<S> df = smul(s.damping * dot(vsub(v1, v0), u), u);
      points[s.a].accumulated_force = vadd(points[s.a].accumulated_force, df);
      points[s.b].accumulated_force = vadd(points[s.b].accumulated_force, smul(S(-1), df));
    }
  }
  void apply_face_forces(const Config<S>& cfg) {  // 629-654
    const S pi = S(PI_F32);
    for (const auto& f : faces) {
      const Point<S> p0 = points[f.v0], p1 = points[f.v1], p2 = points[f.v2];
      const V3<S> avg = vdivs(vadd(vadd(p0.velocity, p1.velocity), p2.velocity), S(3));
      const V3<S> rv = vsub(avg, cfg.wind);
      const S eff = face_area(f) * std::fabs(dot(face_normal(f), rv));
      const V3<S> drag = smul(S(-1) * cfg.drag_coefficient * eff, rv);
      const V3<S> lift =
          smul(S(-1) * cfg.lift_coefficient * eff, vmuls(rv, magnitude(cross(face_normal(f), rv))));
      const V3<S> total = vadd(drag, lift);
      const V3<S> f0 = smul(vertex_angle_k(f, 0) / pi, total);
      const V3<S> f1 = smul(vertex_angle_k(f, 1) / pi, total);
      const V3<S> f2 = smul(vertex_angle_k(f, 2) / pi, total);
      points[f.v0].accumulated_force = vadd(points[f.v0].accumulated_force, f0);
      points[f.v1].accumulated_force = vadd(points[f.v1].accumulated_force, f1);
      points[f.v2].accumulated_force = vadd(points[f.v2].accumulated_force, f2);
    }
  }
  void accumulate_forces(const Config<S>& cfg) {  // 515-525
    apply_external_point_forces(cfg);
    apply_strut_forces();
    apply_face_forces(cfg);
    for (uint64_t pin : pinned_points) points[pin].accumulated_force = zero3<S>();
  }

  void update_points(std::vector<Point<S>> new_points, const std::vector<const CollidableMesh<S>*>& obstacles,
                     const Config<S>& cfg) {  // 423-497
    std::vector<const CFace<S>*> obstacle_faces;
    for (const auto* o : obstacles)
      for (const auto& f : o->faces) obstacle_faces.push_back(&f);
    const S dt_duration = S(duration_roundtrip(cfg.dt));
    const S dt = S(cfg.dt);
    const S eps = S(EPSILON_F32);
    const size_t n = std::min(new_points.size(), points.size());
    for (size_t i = 0; i < n; ++i) {
      Point<S>& np = new_points[i];
      const Point<S>& op = points[i];
      const long hit = collided_face(obstacle_faces, op.position, np.position, dt_duration);
      if (hit < 0) continue;
      const CFace<S>& face = *obstacle_faces[size_t(hit)];
      const S old_d = face.distance_from_plane(op.position);
      const S new_d = face.distance_from_plane(np.position);
      const S fraction = old_d / (old_d - new_d);
      const V3<S> cp = vadd(op.position, smul(dt * fraction, op.velocity));
      const V3<S> vc = vadd(op.velocity, vdivs(smul(dt * fraction, op.accumulated_force), op.mass));
      const V3<S> new_position = vadd(cp, vmuls(face.normal(), eps));
      const V3<S> vcn = smul(dot(vc, face.normal()), face.normal());
      const V3<S> vct = vsub(vc, vcn);
      const V3<S> vrn = vmuls(smul(S(-1), vcn), cfg.coefficient_of_restitution);
      V3<S> vrt;
      if (is_zero(vct) || std::isnan(magnitude(vct))) {
        vrt = zero3<S>();
      } else {
        vrt = vsub(vct, vmuls(normalize(vct), std::fmin(cfg.coefficient_of_friction * magnitude(vcn),
                                                       magnitude(vct))));
      }
      np.position = new_position;
      np.velocity = vadd(vrn, vrt);
    }
    const std::vector<Point<S>> original = points;
    points = std::move(new_points);
    for (uint64_t pin : pinned_points) points[pin] = original[pin];
  }

  void clear_forces() {  // 656-660
    for (auto& p : points) p.accumulated_force = zero3<S>();
  }

  template <class T>
  SpringyMesh<T> widen() const {
    SpringyMesh<T> w;
    for (const auto& s : struts) w.struts.push_back(Strut<T>{T(s.stiffness), T(s.damping), T(s.length), s.a, s.b, s.f0, s.f1});
    w.faces = faces;
    for (const auto& p : points)
      w.points.push_back(Point<T>{T(p.mass), {T(p.position.x), T(p.position.y), T(p.position.z)},
                                  {T(p.velocity.x), T(p.velocity.y), T(p.velocity.z)},
                                  {T(p.accumulated_force.x), T(p.accumulated_force.y), T(p.accumulated_force.z)}});
    w.pinned_points = pinned_points;
    return w;
  }
};

// Cloth::new, cloth.rs:20-113.
static SpringyMesh<float> make_cloth(uint64_t rows, uint64_t cols, float spacing, V3<float> position, float point_mass,
                                     float tk, float tc, float sk, float sc, float bk, float bc,
                                     const std::vector<uint64_t>& pinned) {
  if (rows < 2 || cols < 2) throw std::invalid_argument("Cloth::new needs at least 2 rows and 2 cols");
  std::vector<V3<float>> pos;
  pos.reserve(rows * cols);
  const V3<float> centre{float(cols) / 2.0f * spacing, float(rows) / 2.0f * spacing, 0.0f};
  for (uint64_t r = 0; r < rows; ++r)
    for (uint64_t c = 0; c < cols; ++c) {
      const V3<float> v{float(c) * spacing, float(r) * spacing, 0.0f};
      pos.push_back(vadd(vsub(v, centre), position));
    }
  KeyMap shear;
  std::vector<uint64_t> idx;
  idx.reserve(6 * (rows - 1) * (cols - 1));
  for (uint64_t r = 0; r + 1 < rows; ++r)
    for (uint64_t c = 0; c + 1 < cols; ++c) {
      const uint64_t i = r * cols + c;
      idx.push_back(i + 1); idx.push_back(i + cols); idx.push_back(i);
      shear[strut_key(i + cols, i + 1)] = {sk, sc};
    }
  for (uint64_t r = 1; r < rows; ++r)
    for (uint64_t c = 0; c + 1 < cols; ++c) {
      const uint64_t i = r * cols + c;
      idx.push_back(i - cols + 1); idx.push_back(i + 1); idx.push_back(i);
    }
  SpringyMesh<float> m = SpringyMesh<float>::make(pos, idx, point_mass * float(rows) * float(cols), tk, tc, &shear);
  for (uint64_t p : pinned) m.add_pin(p);
  for (uint64_t r = 0; r + 2 < rows; ++r)
    for (uint64_t c = 0; c + 2 < cols; ++c) {
      const uint64_t i = r * cols + c;
      m.add_strut(i, i + 2, bk, bc);
      m.add_strut(i, i + 2 * cols, bk, bc);
    }
  return m;
}

// Simulation::step, springy/simulation.rs:27-45.
template <class S>
static void simulation_step(std::vector<SpringyMesh<S>*>& meshes, const std::vector<const CollidableMesh<S>*>& obstacles,
                            const Config<S>& cfg) {
  for (SpringyMesh<S>* mesh : meshes) {
    mesh->accumulate_forces(cfg);
    State<S, Point<S>> st;
    st.elements = mesh->points;  // State::new(points.to_vec())
    State<S, Point<S>> next = cfg.integration == 1 ? st.rk4_step(S(cfg.dt)) : st.euler_step(S(cfg.dt));
    mesh->update_points(std::move(next.elements), obstacles, cfg);
    mesh->clear_forces();
  }
}

// ------------------------------------------ state.rs unit-test Stateful types ---
// state.rs:120-164 (a 6-float point under constant acceleration (1,-1,0)) and
// 187-216 (y' = y - t^2 + 1).  Kept here so the State restatement can be
// pinned against the reference's own euler_step / rk4_step assertions.
struct TestPoint {
  V3<float> position, velocity;
  static size_t num_state_elements() { return 6; }
  static TestPoint from_state_vector(const std::vector<float>& d) {
    if (d.size() != 6) throw std::runtime_error("State Vector incorrect size!");
    return TestPoint{{d[0], d[1], d[2]}, {d[3], d[4], d[5]}};
  }
  std::vector<float> derivative() const { return {velocity.x, velocity.y, velocity.z, 1.0f, -1.0f, 0.0f}; }
  std::vector<float> as_state() const { return {position.x, position.y, position.z, velocity.x, velocity.y, velocity.z}; }
};
struct ExampleFn {
  float y, t, timestep;
  static size_t num_state_elements() { return 3; }
  static ExampleFn from_state_vector(const std::vector<float>& d) {
    if (d.size() != 3) throw std::runtime_error("State Vector incorrect size!");
    return ExampleFn{d[0], d[1], d[2]};
  }
  std::vector<float> derivative() const { return {y - std::pow(t, 2.0f) + 1.0f, 1.0f, 0.0f}; }
  std::vector<float> as_state() const { return {y, t, timestep}; }
};

}  // namespace oracle

// =================================================================== C ABI ===
// ctypes surface used by tests/ and bench.py.  Handles are opaque; every
// function returns 0 on success and -1 on error (message: oracle_last_error).

using namespace oracle;

namespace {
thread_local std::string g_err;
struct MeshH {
  int prec;  // 32 or 64
  std::unique_ptr<SpringyMesh<float>> m32;
  std::unique_ptr<SpringyMesh<double>> m64;
};
struct ObsH {
  CollidableMesh<float> o32;
  CollidableMesh<double> o64;
};
struct SimH {
  int prec;
  std::vector<MeshH*> meshes;
  std::vector<ObsH*> obstacles;
  Config<float> c32;
  Config<double> c64;
};
}  // namespace

extern "C" {

typedef struct oracle_config {
  int32_t integration;
  float dt;
  float gravity[3];
  float wind[3];
  float lift_coefficient;
  float drag_coefficient;
  float coefficient_of_restitution;
  float coefficient_of_friction;
} oracle_config;

const char* oracle_last_error(void) { return g_err.c_str(); }

#define ORACLE_TRY(...)                  \
  try {                                  \
    __VA_ARGS__;                         \
    return 0;                            \
  } catch (const std::exception& e) {    \
    g_err = e.what();                    \
    return -1;                           \
  }

static std::vector<V3<float>> to_v3(const float* p, uint64_t n) {
  std::vector<V3<float>> v(n);
  for (uint64_t i = 0; i < n; ++i) v[i] = {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
  return v;
}

}  // extern "C"

template <class S>
static Config<S> to_cfg(const oracle_config* c) {
  if (!(c->dt >= 0.0f) || !std::isfinite(c->dt)) throw std::invalid_argument("dt must be finite and >= 0");
  Config<S> o;
  o.integration = c->integration;
  o.dt = c->dt;
  o.gravity = {S(c->gravity[0]), S(c->gravity[1]), S(c->gravity[2])};
  o.wind = {S(c->wind[0]), S(c->wind[1]), S(c->wind[2])};
  o.lift_coefficient = S(c->lift_coefficient);
  o.drag_coefficient = S(c->drag_coefficient);
  o.coefficient_of_restitution = S(c->coefficient_of_restitution);
  o.coefficient_of_friction = S(c->coefficient_of_friction);
  return o;
}

extern "C" {

// Config::default(), config.rs:20-32.
int oracle_config_default(oracle_config* out) {
  std::memset(out, 0, sizeof(*out));
  out->integration = 1;
  out->dt = 0.001f;  // Duration::from_millis(1).as_secs_f32()
  out->gravity[1] = -10.0f;
  out->lift_coefficient = 1.0f;
  out->drag_coefficient = 1.0f;
  out->coefficient_of_restitution = 0.95f;
  out->coefficient_of_friction = 0.3f;
  return 0;
}

float oracle_duration_roundtrip(float x) { return duration_roundtrip(x); }

int oracle_mesh_new(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, float mass, float k, float c,
                    const uint32_t* ov_ab, const float* ov_kc, uint64_t nov, void** out) {
  ORACLE_TRY({
    std::vector<uint64_t> ix(idx, idx + ni);
    KeyMap ov;
    for (uint64_t i = 0; i < nov; ++i) ov[strut_key(ov_ab[2 * i], ov_ab[2 * i + 1])] = {ov_kc[2 * i], ov_kc[2 * i + 1]};
    auto* h = new MeshH{32, nullptr, nullptr};
    h->m32.reset(new SpringyMesh<float>(SpringyMesh<float>::make(to_v3(pos, nv), ix, mass, k, c, ov_ab ? &ov : nullptr)));
    *out = h;
  })
}

int oracle_cloth_new(uint64_t rows, uint64_t cols, float spacing, const float* position, float point_mass, float tk,
                     float tc, float sk, float sc, float bk, float bc, const uint64_t* pins, uint64_t npins, void** out) {
  ORACLE_TRY({
    std::vector<uint64_t> p(pins, pins + npins);
    auto* h = new MeshH{32, nullptr, nullptr};
    h->m32.reset(new SpringyMesh<float>(
        make_cloth(rows, cols, spacing, {position[0], position[1], position[2]}, point_mass, tk, tc, sk, sc, bk, bc, p)));
    *out = h;
  })
}

int oracle_mesh_widen(void* h32, void** out) {
  ORACLE_TRY({
    auto* h = static_cast<MeshH*>(h32);
    if (h->prec != 32) throw std::invalid_argument("mesh is already f64");
    auto* w = new MeshH{64, nullptr, nullptr};
    w->m64.reset(new SpringyMesh<double>(h->m32->widen<double>()));
    *out = w;
  })
}

int oracle_mesh_free(void* h) {
  delete static_cast<MeshH*>(h);
  return 0;
}

int oracle_mesh_add_strut(void* h, uint64_t a, uint64_t b, float k, float c) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("add_strut on a widened mesh");
    m->m32->add_strut(a, b, k, c);
  })
}

int oracle_mesh_add_struts(void* h, const uint32_t* a, const uint32_t* b, const float* k, const float* c, uint64_t n) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("add_strut on a widened mesh");
    for (uint64_t i = 0; i < n; ++i) m->m32->add_strut(a[i], b[i], k[i], c[i]);
  })
}

int oracle_mesh_add_pins(void* h, const uint32_t* p, uint64_t n) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    for (uint64_t i = 0; i < n; ++i) {
      if (m->prec == 32) m->m32->add_pin(p[i]); else m->m64->add_pin(p[i]);
    }
  })
}

int oracle_mesh_add_pin(void* h, uint64_t i) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec == 32) m->m32->add_pin(i); else m->m64->add_pin(i);
  })
}

int oracle_mesh_counts(void* h, uint64_t* out4) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec == 32) {
      out4[0] = m->m32->points.size(); out4[1] = m->m32->struts.size();
      out4[2] = m->m32->faces.size(); out4[3] = m->m32->pinned_points.size();
    } else {
      out4[0] = m->m64->points.size(); out4[1] = m->m64->struts.size();
      out4[2] = m->m64->faces.size(); out4[3] = m->m64->pinned_points.size();
    }
  })
}

}  // extern "C"

template <class S>
static void get_points_t(const SpringyMesh<S>& m, double* out) {
  for (size_t i = 0; i < m.points.size(); ++i) {
    const auto s = m.points[i].as_state();
    for (int j = 0; j < 10; ++j) out[10 * i + j] = double(s[j]);
  }
}

extern "C" {

// Points in the Stateful::as_state layout [m, p, v, F], as f32 (f32 mesh) or f64.
int oracle_mesh_get_points_f32(void* h, float* out) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 readback of an f64 mesh");
    for (size_t i = 0; i < m->m32->points.size(); ++i) {
      const auto s = m->m32->points[i].as_state();
      std::memcpy(out + 10 * i, s.data(), 10 * sizeof(float));
    }
  })
}
int oracle_mesh_get_points_f64(void* h, double* out) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec == 32) get_points_t(*m->m32, out); else get_points_t(*m->m64, out);
  })
}
int oracle_mesh_set_points_f32(void* h, const float* in) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 write to an f64 mesh");
    for (size_t i = 0; i < m->m32->points.size(); ++i)
      m->m32->points[i] = Point<float>::from_state_vector(std::vector<float>(in + 10 * i, in + 10 * i + 10));
  })
}

int oracle_mesh_get_struts(void* h, float* kcl, uint64_t* ab, int64_t* faces) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 mesh expected");
    const auto& st = m->m32->struts;
    for (size_t i = 0; i < st.size(); ++i) {
      if (kcl) { kcl[3 * i] = st[i].stiffness; kcl[3 * i + 1] = st[i].damping; kcl[3 * i + 2] = st[i].length; }
      if (ab) { ab[2 * i] = st[i].a; ab[2 * i + 1] = st[i].b; }
      if (faces) { faces[2 * i] = st[i].f0; faces[2 * i + 1] = st[i].f1; }
    }
  })
}

// Mirror of the library's fgb_mesh_set_strut_params extension: replace the
// (already length-scaled) per-strut stiffness and damping in strut order.
int oracle_mesh_set_strut_params(void* h, const float* k, const float* c) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 mesh expected");
    for (size_t i = 0; i < m->m32->struts.size(); ++i) {
      m->m32->struts[i].stiffness = k[i];
      m->m32->struts[i].damping = c[i];
    }
  })
}

int oracle_mesh_get_faces(void* h, uint64_t* struts3, uint64_t* verts3) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    const auto& fs = m->prec == 32 ? m->m32->faces : m->m64->faces;
    for (size_t i = 0; i < fs.size(); ++i) {
      if (struts3) { struts3[3 * i] = fs[i].s0; struts3[3 * i + 1] = fs[i].s1; struts3[3 * i + 2] = fs[i].s2; }
      if (verts3) { verts3[3 * i] = fs[i].v0; verts3[3 * i + 1] = fs[i].v1; verts3[3 * i + 2] = fs[i].v2; }
    }
  })
}

int oracle_mesh_get_pins(void* h, uint64_t* out) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    const auto& p = m->prec == 32 ? m->m32->pinned_points : m->m64->pinned_points;
    std::memcpy(out, p.data(), p.size() * sizeof(uint64_t));
  })
}

int oracle_mesh_face_normal(void* h, uint64_t f, float* out3) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    const V3<float> n = m->m32->face_normal(m->m32->faces.at(f));
    out3[0] = n.x; out3[1] = n.y; out3[2] = n.z;
  })
}

int oracle_mesh_face_angle(void* h, uint64_t f, int k, float* out) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    *out = m->m32->vertex_angle_k(m->m32->faces.at(f), k);
  })
}

int oracle_mesh_accumulate_forces(void* h, const oracle_config* cfg) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec == 32) m->m32->accumulate_forces(to_cfg<float>(cfg)); else m->m64->accumulate_forces(to_cfg<double>(cfg));
  })
}

int oracle_mesh_clear_forces(void* h) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec == 32) m->m32->clear_forces(); else m->m64->clear_forces();
  })
}

// State::euler_step / rk4_step on the mesh's current points (integration 0/1);
// writes the new points in the as_state layout (f32 meshes only).
int oracle_mesh_integrate(void* h, int integration, float dt, float* out) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 mesh expected");
    State<float, Point<float>> st;
    st.elements = m->m32->points;
    State<float, Point<float>> nx = integration == 1 ? st.rk4_step(dt) : st.euler_step(dt);
    for (size_t i = 0; i < nx.elements.size(); ++i) {
      const auto s = nx.elements[i].as_state();
      std::memcpy(out + 10 * i, s.data(), 10 * sizeof(float));
    }
  })
}

int oracle_collidable_new(const float* pos, uint64_t nv, const uint32_t* idx, uint64_t ni, void** out) {
  ORACLE_TRY({
    std::vector<uint64_t> ix(idx, idx + ni);
    auto* h = new ObsH();
    h->o32 = CollidableMesh<float>::make(to_v3(pos, nv), ix);
    std::vector<V3<double>> p64;
    for (const auto& v : h->o32.vertices) p64.push_back({double(v.x), double(v.y), double(v.z)});
    for (const auto& f : h->o32.faces)
      h->o64.faces.push_back(CFace<double>{{f.v0.x, f.v0.y, f.v0.z}, {f.v1.x, f.v1.y, f.v1.z}, {f.v2.x, f.v2.y, f.v2.z}});
    h->o64.vertices = p64;
    *out = h;
  })
}
int oracle_collidable_free(void* h) {
  delete static_cast<ObsH*>(h);
  return 0;
}
int oracle_collidable_counts(void* h, uint64_t* out3) {
  ORACLE_TRY({
    auto* o = static_cast<ObsH*>(h);
    out3[0] = o->o32.vertices.size(); out3[1] = o->o32.edges.size(); out3[2] = o->o32.faces.size();
  })
}
int oracle_collidable_get(void* h, float* faces9, float* edges6) {
  ORACLE_TRY({
    auto* o = static_cast<ObsH*>(h);
    for (size_t i = 0; i < o->o32.faces.size() && faces9; ++i) {
      const auto& f = o->o32.faces[i];
      const float v[9] = {f.v0.x, f.v0.y, f.v0.z, f.v1.x, f.v1.y, f.v1.z, f.v2.x, f.v2.y, f.v2.z};
      std::memcpy(faces9 + 9 * i, v, sizeof(v));
    }
    for (size_t i = 0; i < o->o32.edges.size() && edges6; ++i) {
      const auto& e = o->o32.edges[i];
      const float v[6] = {e.first.x, e.first.y, e.first.z, e.second.x, e.second.y, e.second.z};
      std::memcpy(edges6 + 6 * i, v, sizeof(v));
    }
  })
}

// First-hit search over the flattened faces of `obs` for each of n segments
// (old[3n] -> new[3n]); out[i] = flattened face index or -1.
int oracle_collided_faces(void* const* obs, uint64_t nobs, const float* old_p, const float* new_p, uint64_t n,
                          float dt, int64_t* out) {
  ORACLE_TRY({
    std::vector<const CFace<float>*> faces;
    for (uint64_t j = 0; j < nobs; ++j)
      for (const auto& f : static_cast<ObsH*>(obs[j])->o32.faces) faces.push_back(&f);
    const float dd = duration_roundtrip(dt);
    for (uint64_t i = 0; i < n; ++i)
      out[i] = collided_face<float>(faces, {old_p[3 * i], old_p[3 * i + 1], old_p[3 * i + 2]},
                                    {new_p[3 * i], new_p[3 * i + 1], new_p[3 * i + 2]}, dd);
  })
}

// SpringyMesh::update_points with host-provided new points (as_state layout).
int oracle_mesh_update_points(void* h, const float* new_points, void* const* obs, uint64_t nobs,
                              const oracle_config* cfg) {
  ORACLE_TRY({
    auto* m = static_cast<MeshH*>(h);
    if (m->prec != 32) throw std::invalid_argument("f32 mesh expected");
    std::vector<Point<float>> np;
    for (size_t i = 0; i < m->m32->points.size(); ++i)
      np.push_back(Point<float>::from_state_vector(std::vector<float>(new_points + 10 * i, new_points + 10 * i + 10)));
    std::vector<const CollidableMesh<float>*> o;
    for (uint64_t j = 0; j < nobs; ++j) o.push_back(&static_cast<ObsH*>(obs[j])->o32);
    m->m32->update_points(std::move(np), o, to_cfg<float>(cfg));
  })
}

// Simulation::new(meshes, obstacles) with Config::default(); all meshes must
// share one precision.
int oracle_sim_new(void* const* meshes, uint64_t nm, void* const* obs, uint64_t nobs, void** out) {
  ORACLE_TRY({
    auto* s = new SimH();
    s->prec = nm ? static_cast<MeshH*>(meshes[0])->prec : 32;
    for (uint64_t i = 0; i < nm; ++i) {
      auto* m = static_cast<MeshH*>(meshes[i]);
      if (m->prec != s->prec) { delete s; throw std::invalid_argument("mixed mesh precisions"); }
      s->meshes.push_back(m);
    }
    for (uint64_t j = 0; j < nobs; ++j) s->obstacles.push_back(static_cast<ObsH*>(obs[j]));
    oracle_config d;
    oracle_config_default(&d);
    s->c32 = to_cfg<float>(&d);
    s->c64 = to_cfg<double>(&d);
    *out = s;
  })
}
int oracle_sim_free(void* h) {
  delete static_cast<SimH*>(h);
  return 0;
}
int oracle_sim_set_config(void* h, const oracle_config* cfg) {
  ORACLE_TRY({
    auto* s = static_cast<SimH*>(h);
    s->c32 = to_cfg<float>(cfg);
    s->c64 = to_cfg<double>(cfg);
  })
}
int oracle_sim_step(void* h, uint64_t nsteps) {
  ORACLE_TRY({
    auto* s = static_cast<SimH*>(h);
    if (s->prec == 32) {
      std::vector<SpringyMesh<float>*> ms;
      for (auto* m : s->meshes) ms.push_back(m->m32.get());
      std::vector<const CollidableMesh<float>*> os;
      for (auto* o : s->obstacles) os.push_back(&o->o32);
      for (uint64_t i = 0; i < nsteps; ++i) simulation_step(ms, os, s->c32);
    } else {
      std::vector<SpringyMesh<double>*> ms;
      for (auto* m : s->meshes) ms.push_back(m->m64.get());
      std::vector<const CollidableMesh<double>*> os;
      for (auto* o : s->obstacles) os.push_back(&o->o64);
      for (uint64_t i = 0; i < nsteps; ++i) simulation_step(ms, os, s->c64);
    }
  })
}

// state.rs:166-185 (euler_step test) and 218-280 (rk4_step test) drivers.
int oracle_state_test_euler(const float* pv6, float h, float* out6) {
  ORACLE_TRY({
    State<float, TestPoint> st;
    st.elements.push_back(TestPoint::from_state_vector(std::vector<float>(pv6, pv6 + 6)));
    auto nx = st.euler_step(h);
    const auto s = nx.elements[0].as_state();
    std::memcpy(out6, s.data(), 6 * sizeof(float));
  })
}
int oracle_state_test_rk4(const float* yth, float h, float* out3) {
  ORACLE_TRY({
    State<float, ExampleFn> st;
    st.elements.push_back(ExampleFn::from_state_vector(std::vector<float>(yth, yth + 3)));
    auto nx = st.rk4_step(h);
    const auto s = nx.elements[0].as_state();
    std::memcpy(out3, s.data(), 3 * sizeof(float));
  })
}

}  // extern "C"
