// Batch replay renderer (declared in include/gbr_replay.h).
//
// Keyframes (gfx/replay/Keyframe.h:70-91) are parsed from the Recorder's
// JSON (io/JsonEspTypes.cpp:102-201) and applied by a Player per environment
// (gfx/replay/Player.cpp:189-370) through the batch player
// (sim/BatchPlayerImplementation.cpp:51-170): instances become node
// hierarchies of the environment's scene, state updates write the root
// node's local transform, deletions clear the scene and re-create the
// remaining instances, light setups become empty nodes carrying lights.
//
// The small linear algebra (quaternion -> matrix, rotation between two
// vectors, 4x4 inverse by Laplace expansion of 2x2 minors, the pinhole and
// orthographic projections) is written out operation by operation, each a
// single float rounding in source order; the oracle's replay restates the
// same sequence.
#include "replay.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>

#include "renderer.h"
#include "trace.h"

namespace gbr {
namespace replay {

namespace {

bool read_floats(const Json* j, float* out, size_t n) {
  if (!j || j->type != Json::Array || j->size() != n) return false;
  for (size_t i = 0; i < n; ++i) {
    if ((*j)[i].type != Json::Number) return false;
    out[i] = float((*j)[i].num);
  }
  return true;
}

bool read_quat(const Json* j, Quat& q) {  // serialized as [w, x, y, z]
  float v[4];
  if (!read_floats(j, v, 4)) return false;
  q.w = v[0];
  q.x = v[1];
  q.y = v[2];
  q.z = v[3];
  return true;
}

bool read_int(const Json* j, int& out) {
  if (!j || j->type != Json::Number) return false;
  out = int(j->num);
  return true;
}

bool read_bool(const Json& obj, const char* key) {
  const Json* j = obj.get(key);
  return j && j->type == Json::Bool && j->b;
}

bool read_transform(const Json* j, Transform& t) {
  if (!j || j->type != Json::Object) return false;
  return read_floats(j->get("translation"), t.translation, 3) && read_quat(j->get("rotation"), t.rotation);
}

std::string lower(std::string s) {
  for (auto& c : s) c = char(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void cross3(const float a[3], const float b[3], float out[3]) {
  out[0] = a[1] * b[2] - a[2] * b[1];
  out[1] = a[2] * b[0] - a[0] * b[2];
  out[2] = a[0] * b[1] - a[1] * b[0];
}

void normalize3(float v[3]) {
  const float len = std::sqrt(dot3(v, v));
  v[0] = v[0] / len;
  v[1] = v[1] / len;
  v[2] = v[2] / len;
}

// Primitive assets the batch renderer can't load (BatchPlayerImplementation.cpp:14-40).
bool supported_asset(const std::string& path) {
  static const char* const prefixes[] = {
      "capsule3DSolid", "capsule3DWireframe", "coneSolid",          "coneWireframe",
      "cubeSolid",      "cubeWireframe",      "cylinderSolid",      "cylinderWireframe",
      "icosphereSolid", "icosphereWireframe", "uvSphereSolid",      "uvSphereWireframe"};
  for (const char* p : prefixes)
    if (path.compare(0, std::strlen(p), p) == 0) return false;
  return true;
}

// Player.cpp:23-33: material overrides are appended to the path after '?'.
std::string strip_override(const std::string& path, bool& stripped) {
  const size_t q = path.find('?');
  stripped = q != std::string::npos;
  return stripped ? path.substr(0, q) : path;
}

gbr_status fail(gbr_status s, const std::string& msg) {
  set_last_error(msg);
  return s;
}

}  // namespace

// ------------------------------------------------------------------ JSON
bool parse_keyframe(const Json& obj, Keyframe& k, std::string& err) {
  if (obj.type != Json::Object) { err = "keyframe is not an object"; return false; }
  if (const Json* loads = obj.get("loads")) {
    for (size_t i = 0; i < loads->size(); ++i) {
      const Json& l = (*loads)[i];
      AssetInfo a;
      read_int(l.get("type"), a.type);
      const Json* fp = l.get("filepath");
      if (!fp || fp->type != Json::String) { err = "load without filepath"; return false; }
      a.filepath = fp->str;
      if (const Json* fr = l.get("frame")) {
        if (!read_floats(fr->get("up"), a.up, 3) || !read_floats(fr->get("front"), a.front, 3)) {
          err = "bad frame of " + a.filepath;
          return false;
        }
        read_floats(fr->get("origin"), a.origin, 3);
      }
      k.loads.push_back(std::move(a));
    }
  }
  if (const Json* cs = obj.get("creations")) {
    for (size_t i = 0; i < cs->size(); ++i) {
      const Json& p = (*cs)[i];
      int key;
      const Json* c = p.get("creation");
      if (!read_int(p.get("instanceKey"), key) || !c || c->type != Json::Object) {
        err = "bad creation entry";
        return false;
      }
      Creation cr;
      const Json* fp = c->get("filepath");
      if (!fp || fp->type != Json::String) { err = "creation without filepath"; return false; }
      cr.filepath = fp->str;
      if (const Json* s = c->get("scale")) {
        if (s->type != Json::Null) {
          if (!read_floats(s, cr.scale, 3)) { err = "bad creation scale"; return false; }
          cr.has_scale = true;
        }
      }
      cr.flags = (read_bool(*c, "isStatic") ? 1u : 0u) | (read_bool(*c, "isRGBD") ? 2u : 0u) |
                 (read_bool(*c, "isSemantic") ? 4u : 0u) |
                 (read_bool(*c, "isTextureSemantic") ? 8u : 0u);
      if (const Json* lk = c->get("lightSetupKey"))
        if (lk->type == Json::String) cr.light_setup_key = lk->str;
      read_int(c->get("rigId"), cr.rig_id);
      k.creations.emplace_back(key, std::move(cr));
    }
  }
  if (const Json* ds = obj.get("deletions")) {
    for (size_t i = 0; i < ds->size(); ++i) {
      int key;
      if (!read_int(&(*ds)[i], key)) { err = "bad deletion"; return false; }
      k.deletions.push_back(key);
    }
  }
  if (const Json* us = obj.get("stateUpdates")) {
    for (size_t i = 0; i < us->size(); ++i) {
      const Json& u = (*us)[i];
      int key;
      const Json* st = u.get("state");
      Transform t;
      if (!read_int(u.get("instanceKey"), key) || !st || !read_transform(st->get("absTransform"), t)) {
        err = "bad state update";
        return false;
      }
      k.state_updates.emplace_back(key, t);
    }
  }
  if (const Json* ms = obj.get("metadata")) {
    for (size_t i = 0; i < ms->size(); ++i) {
      const Json& m = (*ms)[i];
      int key;
      const Json* md = m.get("metadata");
      Metadata d;
      if (!read_int(m.get("instanceKey"), key) || !md || !read_int(md->get("objectId"), d.object_id) ||
          !read_int(md->get("semanticId"), d.semantic_id)) {
        err = "bad metadata entry";
        return false;
      }
      k.metadata.emplace_back(key, d);
    }
  }
  // rigCreations / rigUpdates: the batch player doesn't implement rigs
  // (BatchPlayerImplementation.cpp:171-186); they are accepted and ignored.
  if (const Json* ut = obj.get("userTransforms")) {
    for (size_t i = 0; i < ut->size(); ++i) {
      const Json& u = (*ut)[i];
      const Json* name = u.get("name");
      Transform t;
      if (!name || name->type != Json::String || !read_transform(u.get("transform"), t)) {
        err = "bad user transform";
        return false;
      }
      k.user_transforms[name->str] = t;
    }
  }
  k.lights_changed = read_bool(obj, "lightsChanged");
  if (k.lights_changed) {
    if (const Json* ls = obj.get("lights")) {
      for (size_t i = 0; i < ls->size(); ++i) {
        const Json& l = (*ls)[i];
        Light li;
        if (!read_floats(l.get("vector"), li.vector, 4) || !read_floats(l.get("color"), li.color, 3)) {
          err = "bad light";
          return false;
        }
        if (const Json* m = l.get("model")) {
          const std::string model = lower(m->str);
          if (model != "global" && model != "camera" && model != "object") {
            err = "Illegal model value '" + m->str + "' specified in JSON to be used to set LightInfo.model";
            return false;
          }
          li.global = model == "global";
        }
        k.lights.push_back(li);
      }
    }
  }
  return true;
}

// ------------------------------------------------------------------ math
void quat_to_matrix(const Quat& q, float m[9]) {
  const float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  const float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
  const float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
  m[0] = 1.0f - 2.0f * (yy + zz);
  m[1] = 2.0f * (xy + wz);
  m[2] = 2.0f * (xz - wy);
  m[3] = 2.0f * (xy - wz);
  m[4] = 1.0f - 2.0f * (xx + zz);
  m[5] = 2.0f * (yz + wx);
  m[6] = 2.0f * (xz + wy);
  m[7] = 2.0f * (yz - wx);
  m[8] = 1.0f - 2.0f * (xx + yy);
}

Quat quat_between(const float a[3], const float b[3]) {
  const float c = dot3(a, b);
  float axis[3];
  if (c < -1.0f + 1.1920929e-07f) {  // opposite: any axis perpendicular to a
    const float x[3] = {1, 0, 0}, y[3] = {0, 1, 0};
    cross3(x, a, axis);
    if (dot3(axis, axis) < 1.1920929e-07f) cross3(y, a, axis);
    normalize3(axis);
    return {axis[0], axis[1], axis[2], 0.0f};
  }
  cross3(a, b, axis);
  const float s = std::sqrt((1.0f + c) * 2.0f);
  const float inv = 1.0f / s;
  return {axis[0] * inv, axis[1] * inv, axis[2] * inv, s * 0.5f};
}

Quat quat_mul(const Quat& a, const Quat& b) {
  const float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
  float c[3];
  cross3(av, bv, c);
  return {a.w * b.x + b.w * a.x + c[0], a.w * b.y + b.w * a.y + c[1], a.w * b.z + b.w * a.z + c[2],
          a.w * b.w - dot3(av, bv)};
}

Quat quat_normalized(const Quat& q) {
  const float len = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return {q.x / len, q.y / len, q.z / len, q.w / len};
}

void quat_rotate(const Quat& q, const float v[3], float out[3]) {
  const float qv[3] = {q.x, q.y, q.z};
  float t[3], c[3];
  cross3(qv, v, t);
  t[0] = 2.0f * t[0];
  t[1] = 2.0f * t[1];
  t[2] = 2.0f * t[2];
  cross3(qv, t, c);
  for (int i = 0; i < 3; ++i) out[i] = v[i] + q.w * t[i] + c[i];
}

Quat frame_to_world(const float up[3], const float front[3]) {
  const float y[3] = {0, 1, 0}, f0[3] = {0, 0, -1};
  const Quat r_up = quat_between(y, up);
  float f[3];
  quat_rotate(r_up, f0, f);
  const Quat w2f = quat_normalized(quat_mul(quat_between(f, front), r_up));
  return {-w2f.x, -w2f.y, -w2f.z, w2f.w};
}

void rigid_matrix(const Quat& q, const float t[3], float m[16]) {
  float r[9];
  quat_to_matrix(q, r);
  for (int c = 0; c < 3; ++c) {
    for (int i = 0; i < 3; ++i) m[c * 4 + i] = r[c * 3 + i];
    m[c * 4 + 3] = 0.0f;
  }
  m[12] = t[0];
  m[13] = t[1];
  m[14] = t[2];
  m[15] = 1.0f;
}

// Inverse by Laplace expansion in 2x2 minors of the top two and bottom two
// rows (D. Eberly, "The Laplace Expansion Theorem: Computing the
// Determinants and Inverses of Matrices", Geometric Tools, 2008).
bool invert4(const float m[16], float out[16]) {
  auto a = [&](int r, int c) { return m[c * 4 + r]; };
  const float s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1);
  const float s1 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
  const float s2 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3);
  const float s3 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
  const float s4 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3);
  const float s5 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
  const float c5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3);
  const float c4 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
  const float c3 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2);
  const float c2 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
  const float c1 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2);
  const float c0 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
  const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
  if (det == 0.0f || !std::isfinite(det)) return false;
  const float inv = 1.0f / det;
  float b[4][4];  // b[row][col]
  b[0][0] = (a(1, 1) * c5 - a(1, 2) * c4 + a(1, 3) * c3) * inv;
  b[0][1] = (-a(0, 1) * c5 + a(0, 2) * c4 - a(0, 3) * c3) * inv;
  b[0][2] = (a(3, 1) * s5 - a(3, 2) * s4 + a(3, 3) * s3) * inv;
  b[0][3] = (-a(2, 1) * s5 + a(2, 2) * s4 - a(2, 3) * s3) * inv;
  b[1][0] = (-a(1, 0) * c5 + a(1, 2) * c2 - a(1, 3) * c1) * inv;
  b[1][1] = (a(0, 0) * c5 - a(0, 2) * c2 + a(0, 3) * c1) * inv;
  b[1][2] = (-a(3, 0) * s5 + a(3, 2) * s2 - a(3, 3) * s1) * inv;
  b[1][3] = (a(2, 0) * s5 - a(2, 2) * s2 + a(2, 3) * s1) * inv;
  b[2][0] = (a(1, 0) * c4 - a(1, 1) * c2 + a(1, 3) * c0) * inv;
  b[2][1] = (-a(0, 0) * c4 + a(0, 1) * c2 - a(0, 3) * c0) * inv;
  b[2][2] = (a(3, 0) * s4 - a(3, 1) * s2 + a(3, 3) * s0) * inv;
  b[2][3] = (-a(2, 0) * s4 + a(2, 1) * s2 - a(2, 3) * s0) * inv;
  b[3][0] = (-a(1, 0) * c3 + a(1, 1) * c1 - a(1, 2) * c0) * inv;
  b[3][1] = (a(0, 0) * c3 - a(0, 1) * c1 + a(0, 2) * c0) * inv;
  b[3][2] = (-a(3, 0) * s3 + a(3, 1) * s1 - a(3, 2) * s0) * inv;
  b[3][3] = (a(2, 0) * s3 - a(2, 1) * s1 + a(2, 2) * s0) * inv;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[c * 4 + r] = b[r][c];
  return true;
}

void sensor_projection(const gbr_replay_config& c, float p[16]) {
  std::memset(p, 0, 16 * sizeof(float));
  const float aspect = float(c.resolution[0]) / float(c.resolution[1]);  // height / width
  const float n = c.near_plane, f = c.far_plane;
  if (c.orthographic) {
    const float sx = 1.0f / c.ortho_scale, sy = aspect / c.ortho_scale;
    const float zs = 2.0f / (n - f);
    p[0] = 2.0f / sx;
    p[5] = 2.0f / sy;
    p[10] = zs;
    p[14] = (n + f) / (n - f);
    p[15] = 1.0f;
    return;
  }
  const float rad = c.hfov_degrees * 3.14159265358979323846f / 180.0f;
  const float t = float(std::tan(double(0.5f * rad)));
  const float scale = 1.0f / (2.0f * n * t);
  const float sx = 1.0f / scale, sy = aspect / scale;
  const float zs = 1.0f / (n - f);
  p[0] = 2.0f * n / sx;
  p[5] = 2.0f * n / sy;
  p[10] = (f + n) * zs;
  p[11] = -1.0f;
  p[14] = 2.0f * f * n * zs;
}

// --------------------------------------------------------------- player impl
void BatchPlayer::warn(const std::string& msg) const {
  if (!quiet_) std::fprintf(stderr, "gbr replay: %s\n", msg.c_str());
}

gbr_status BatchPlayer::load_and_create(const AssetInfo& info, const Creation& c, uint64_t* node) {
  *node = 0;
  if (!supported_asset(c.filepath)) {
    warn("Unsupported render asset: " + c.filepath);
    return GBR_OK;
  }
  if (!r_.has_hierarchy(c.filepath.c_str())) {
    warn(c.filepath + " not found in any composite file, loading from the filesystem");
    if (gbr_status s = r_.add_file(c.filepath.c_str(), GBR_FILE_WHOLE | GBR_FILE_GENERATE_MIPMAP, nullptr))
      return fail(s, "addFile failed for " + c.filepath + ": " + last_error_cstr());
    if (!r_.has_hierarchy(c.filepath.c_str()))
      return fail(GBR_ERROR_NOT_FOUND, "no hierarchy named " + c.filepath + " after loading it");
  }
  // Bake = scaling(scale) * rotation(frame to world) (BatchPlayerImplementation.cpp:78-85).
  float r[9];
  quat_to_matrix(frame_to_world(info.up, info.front), r);
  const float one[3] = {1, 1, 1};
  const float* s = c.has_scale ? c.scale : one;
  float bake[16] = {};
  for (int col = 0; col < 3; ++col)
    for (int row = 0; row < 3; ++row) bake[col * 4 + row] = s[row] * r[col * 3 + row];
  bake[15] = 1.0f;
  uint64_t id;
  if (gbr_status st = r_.add_node_hierarchy(scene_, c.filepath.c_str(), bake, &id)) return st;
  *node = id + 1;
  return GBR_OK;
}

gbr_status BatchPlayer::delete_all() { return r_.clear(scene_); }

gbr_status BatchPlayer::set_matrix(uint64_t node, const float m[16]) {
  float* t;
  uint64_t n;
  if (gbr_status s = r_.transformations(scene_, &t, &n)) return s;
  if (node == 0 || node > n) return fail(GBR_ERROR_INVALID_ARGUMENT, "replay: bad node handle");
  std::memcpy(t + (node - 1) * 16, m, 16 * sizeof(float));
  return GBR_OK;
}

gbr_status BatchPlayer::set_transform(uint64_t node, const Transform& tr) {
  float m[16];
  rigid_matrix(tr.rotation, tr.translation, m);
  return set_matrix(node, m);
}

gbr_status BatchPlayer::get_matrix(uint64_t node, float m[16]) const {
  float* t;
  uint64_t n;
  if (gbr_status s = r_.transformations(scene_, &t, &n)) return s;
  if (node == 0 || node > n) return fail(GBR_ERROR_INVALID_ARGUMENT, "replay: bad node handle");
  std::memcpy(m, t + (node - 1) * 16, 16 * sizeof(float));
  return GBR_OK;
}

// The reference's batch player ignores instance metadata
// (AbstractPlayerImplementation::setNodeMetadata is empty); here a defined
// semantic id goes to the semantic plane of the instance's draws.
gbr_status BatchPlayer::set_metadata(uint64_t node, const Metadata& md) {
  if (node == 0 || md.semantic_id < 0) return GBR_OK;
  return r_.set_semantic_id(scene_, node - 1, uint32_t(md.semantic_id));
}

// BatchPlayerImplementation::changeLightSetup (:129-169).
gbr_status BatchPlayer::change_lights(const std::vector<Light>& lights) {
  if (r_.config().max_light_count == 0) {
    warn("Attempted to change " + std::to_string(lights.size()) + " lights for scene " +
         std::to_string(scene_) + " but the renderer is configured without lights");
    return GBR_OK;
  }
  if (gbr_status s = r_.clear_lights(scene_)) return s;
  for (const Light& l : lights) {
    if (!l.global)
      return fail(GBR_ERROR_INVALID_ARGUMENT, "replay: only lights in the global position model are supported");
    uint64_t node, id;
    if (gbr_status s = r_.add_empty_node(scene_, &node)) return s;
    float m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    uint32_t type;
    if (l.vector[3] != 0.0f) {
      m[12] = l.vector[0];
      m[13] = l.vector[1];
      m[14] = l.vector[2];
      type = GBR_LIGHT_POINT;
    } else {
      // lookAt(origin, vector, +Y): columns right, up, backward.  NaN when
      // the vector is along Y, as the reference; only the backward column
      // (the light direction) is used.
      float back[3] = {0.0f - l.vector[0], 0.0f - l.vector[1], 0.0f - l.vector[2]};
      normalize3(back);
      const float up[3] = {0, 1, 0};
      float right[3], real_up[3];
      cross3(up, back, right);
      normalize3(right);
      cross3(back, right, real_up);
      for (int i = 0; i < 3; ++i) {
        m[i] = right[i];
        m[4 + i] = real_up[i];
        m[8 + i] = back[i];
      }
      type = GBR_LIGHT_DIRECTIONAL;
    }
    if (gbr_status s = set_matrix(node + 1, m)) return s;
    if (gbr_status s = r_.add_light(scene_, node, type, &id)) return s;
    float* colors;
    uint64_t n;
    if (gbr_status s = r_.light_colors(scene_, &colors, &n)) return s;
    std::memcpy(colors + id * 3, l.color, 3 * sizeof(float));
  }
  return GBR_OK;
}

// ------------------------------------------------------------------ player
void Player::set_keyframes(std::vector<Keyframe> k) {
  keyframes_ = std::move(k);
}

gbr_status Player::set_single_keyframe(Keyframe k) {
  keyframes_.clear();
  index_ = -1;
  keyframes_.push_back(std::move(k));
  return set_keyframe_index(0);
}

gbr_status Player::set_keyframe_index(int index) {
  if (index < -1 || index >= keyframe_count())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "setKeyframeIndex: index " + std::to_string(index) +
                                                " out of range for " + std::to_string(keyframe_count()) +
                                                " keyframes");
  if (index < index_)
    if (gbr_status s = clear_frame()) return s;
  while (index_ < index)
    if (gbr_status s = apply(keyframes_[size_t(++index_)])) return s;
  return GBR_OK;
}

const Transform* Player::user_transform(const std::string& name) const {
  if (index_ < 0 || index_ >= keyframe_count()) return nullptr;
  const auto& u = keyframes_[size_t(index_)].user_transforms;
  auto it = u.find(name);
  return it == u.end() ? nullptr : &it->second;
}

gbr_status Player::close() {
  gbr_status s = clear_frame();
  keyframes_.clear();
  return s;
}

gbr_status Player::clear_frame() {
  gbr_status s = impl_.delete_all();
  created_.clear();
  asset_infos_.clear();
  records_.clear();
  index_ = -1;
  return s;
}

gbr_status Player::apply(const Keyframe& k) {
  for (const AssetInfo& a : k.loads) {
    if (failed_.count(a.filepath)) continue;
    asset_infos_[a.filepath] = a;
  }
  for (const auto& pc : k.creations) {
    bool stripped;
    Creation c = pc.second;
    c.filepath = strip_override(pc.second.filepath, stripped);
    if (stripped) impl_.warn("Ignoring material-override for [" + pc.second.filepath + "]");
    auto info = asset_infos_.find(c.filepath);
    if (info == asset_infos_.end()) {
      if (failed_.insert(c.filepath).second) impl_.warn("Missing asset info for [" + c.filepath + "]");
      continue;
    }
    uint64_t node;
    if (gbr_status s = impl_.load_and_create(info->second, c, &node)) return s;
    if (!node) {
      if (failed_.insert(c.filepath).second) impl_.warn("Load failed for asset [" + c.filepath + "]");
      continue;
    }
    if (created_.count(pc.first))
      return fail(GBR_ERROR_INVALID_ARGUMENT, "replay: instance key " + std::to_string(pc.first) +
                                                  " created twice");
    created_[pc.first] = node;
    records_[pc.first] = Record{c, Metadata()};
  }
  for (const auto& pm : k.metadata) {
    auto it = created_.find(pm.first);
    if (it == created_.end()) continue;
    if (gbr_status s = impl_.set_metadata(it->second, pm.second)) return s;
    records_[pm.first].metadata = pm.second;
  }
  if (gbr_status s = process_deletions(k)) return s;
  for (const auto& pu : k.state_updates) {
    auto it = created_.find(pu.first);
    if (it == created_.end()) continue;
    if (gbr_status s = impl_.set_transform(it->second, pu.second)) return s;
  }
  if (k.lights_changed)
    if (gbr_status s = impl_.change_lights(k.lights)) return s;
  return GBR_OK;
}

// Player::hackProcessDeletions, batch branch (Player.cpp:300-357): the scene
// is cleared and every remaining instance re-created (in instance-key
// order) with its metadata and latest transform.
gbr_status Player::process_deletions(const Keyframe& k) {
  if (k.deletions.empty()) return GBR_OK;
  std::map<int, std::array<float, 16>> latest;
  for (const auto& pc : created_)
    if (gbr_status s = impl_.get_matrix(pc.second, latest[pc.first].data())) return s;
  if (gbr_status s = impl_.delete_all()) return s;
  for (int key : k.deletions) {
    auto it = created_.find(key);
    if (it == created_.end()) continue;
    created_.erase(it);
    records_.erase(key);
  }
  for (auto& pc : created_) {
    const Record& rec = records_[pc.first];
    uint64_t node;
    if (gbr_status s = impl_.load_and_create(asset_infos_[rec.creation.filepath], rec.creation, &node))
      return s;
    if (!node) return fail(GBR_ERROR_STATE, "replay: re-creating " + rec.creation.filepath + " failed");
    if (gbr_status s = impl_.set_metadata(node, rec.metadata)) return s;
    pc.second = node;
    if (gbr_status s = impl_.set_matrix(node, latest[pc.first].data())) return s;
  }
  return GBR_OK;
}

// ---------------------------------------------------------------- renderer
ReplayRenderer* ReplayRenderer::create(const gbr_replay_config& c, gbr_status& st) {
  st = GBR_ERROR_INVALID_ARGUMENT;
  if (c.num_environments == 0) { set_last_error("ReplayRenderer: num_environments must be positive"); return nullptr; }
  if (!c.standalone) {
    st = GBR_ERROR_STATE;
    set_last_error("BatchReplayRenderer: only the standalone renderer exists (no GL framebuffer to draw into)");
    return nullptr;
  }
  if (c.resolution[0] <= 0 || c.resolution[1] <= 0 || c.resolution[0] > 16384 || c.resolution[1] > 16384) {
    set_last_error("ReplayRenderer: bad sensor resolution");
    return nullptr;
  }
  if (!(c.near_plane > 0.0f) || !(c.far_plane > c.near_plane) ||
      (!c.orthographic && !(c.hfov_degrees > 0.0f && c.hfov_degrees < 180.0f)) ||
      (c.orthographic && !(c.ortho_scale > 0.0f))) {
    set_last_error("ReplayRenderer: bad sensor projection parameters");
    return nullptr;
  }
  std::unique_ptr<ReplayRenderer> rr(new ReplayRenderer());
  rr->cfg_ = c;
  rr->sensor_name_ = c.sensor_uuid ? c.sensor_uuid : "rgba_camera";
  rr->cfg_.sensor_uuid = nullptr;
  sensor_projection(c, rr->projection_);
  gbr_replay_environment_grid_size(int32_t(c.num_environments), rr->grid_);
  gbr_config rc;
  gbr_config_init(&rc);
  rc.tile_size[0] = c.resolution[1];
  rc.tile_size[1] = c.resolution[0];
  rc.tile_count[0] = rr->grid_[0];
  rc.tile_count[1] = rr->grid_[1];
  rc.max_light_count = c.max_light_count;
  rc.ambient_factor = c.ambient_factor;
  rc.cuda_device = c.gpu_device_id;
  rc.standalone_flags = c.quiet ? GBR_STANDALONE_QUIET_LOG : 0u;
  rc.draw_mode = c.draw_mode;
  std::string err;
  rr->renderer_ = Renderer::create(rc, err);
  if (!rr->renderer_) {
    set_last_error(err);
    st = err.find("memory") != std::string::npos ? GBR_ERROR_OUT_OF_MEMORY
         : err.find("cuda") != std::string::npos  ? GBR_ERROR_CUDA
                                                  : GBR_ERROR_INVALID_ARGUMENT;
    return nullptr;
  }
  for (uint32_t i = 0; i < c.num_environments; ++i)
    rr->players_.emplace_back(new Player(BatchPlayer(*rr->renderer_, i, c.quiet != 0)));
  std::array<float, 16> id{};
  id[0] = id[5] = id[10] = id[15] = 1.0f;
  rr->camera_.assign(c.num_environments, id);
  st = GBR_OK;
  return rr.release();
}

ReplayRenderer::~ReplayRenderer() { close(); }

gbr_status ReplayRenderer::close() {
  if (!renderer_) return GBR_OK;
  for (auto& p : players_) p->close();
  players_.clear();
  renderer_->release();
  renderer_ = nullptr;
  return GBR_OK;
}

gbr_status ReplayRenderer::check_env(uint32_t env, const char* fn) const {
  if (!renderer_) return fail(GBR_ERROR_STATE, std::string(fn) + ": the replay renderer is closed");
  if (env >= players_.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, std::string(fn) + ": envIndex " + std::to_string(env) +
                                                " is out of range");
  return GBR_OK;
}

gbr_status ReplayRenderer::preload_file(const char* filename) {
  if (!renderer_) return fail(GBR_ERROR_STATE, "preloadFile: the replay renderer is closed");
  return renderer_->add_file(filename, 0, nullptr);
}

gbr_status ReplayRenderer::clear_environment(uint32_t env) {
  if (gbr_status s = check_env(env, "clearEnvironment")) return s;
  return players_[env]->close();
}

gbr_status ReplayRenderer::set_keyframe_json(uint32_t env, const char* json, uint64_t n, bool wrapped) {
  TraceRange trace_("replay.set_keyframe");
  if (gbr_status s = check_env(env, "setEnvironmentKeyframe")) return s;
  Json doc;
  JsonParser jp{json, json + n, {}};
  if (!jp.parse(doc)) return fail(GBR_ERROR_INVALID_ARGUMENT, "setEnvironmentKeyframe: bad JSON: " + jp.err);
  const Json* obj = &doc;
  if (wrapped) {
    obj = doc.get("keyframe");
    if (!obj) return fail(GBR_ERROR_INVALID_ARGUMENT, "setEnvironmentKeyframe: no \"keyframe\" member");
  }
  Keyframe k;
  std::string err;
  if (!parse_keyframe(*obj, k, err)) return fail(GBR_ERROR_INVALID_ARGUMENT, "setEnvironmentKeyframe: " + err);
  return players_[env]->set_single_keyframe(std::move(k));
}

gbr_status ReplayRenderer::set_keyframes_json(uint32_t env, const char* json, uint64_t n) {
  if (gbr_status s = check_env(env, "readKeyframes")) return s;
  Json doc;
  JsonParser jp{json, json + n, {}};
  if (!jp.parse(doc)) return fail(GBR_ERROR_INVALID_ARGUMENT, "readKeyframes: bad JSON: " + jp.err);
  const Json* arr = doc.get("keyframes");
  if (!arr || arr->type != Json::Array)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "readKeyframes: no \"keyframes\" array");
  std::vector<Keyframe> ks(arr->size());
  for (size_t i = 0; i < arr->size(); ++i) {
    std::string err;
    if (!parse_keyframe((*arr)[i], ks[i], err))
      return fail(GBR_ERROR_INVALID_ARGUMENT, "readKeyframes: keyframe " + std::to_string(i) + ": " + err);
  }
  if (gbr_status s = players_[env]->close()) return s;
  players_[env]->set_keyframes(std::move(ks));
  return GBR_OK;
}

// setEnvironmentKeyframe (+ setSensorTransformsFromKeyframe) for environments
// first .. first + count - 1 in one call.  Every document is parsed before any
// is applied, so a malformed one leaves all environments unchanged; large
// batches are parsed on several host threads (the parser keeps no shared
// state).  The keyframes are then applied in environment order, exactly as
// the per-environment calls would.
gbr_status ReplayRenderer::set_keyframe_batch(uint32_t first, uint32_t count, const char* const* json,
                                              const uint64_t* length, const char* sensor_prefix) {
  TraceRange trace_("replay.set_keyframes_batch");
  if (!renderer_) return fail(GBR_ERROR_STATE, "setEnvironmentKeyframes: the replay renderer is closed");
  if (uint64_t(first) + count > players_.size())
    return fail(GBR_ERROR_INVALID_ARGUMENT, "setEnvironmentKeyframes: environments " + std::to_string(first) +
                                                " + " + std::to_string(count) + " exceed the environment count " +
                                                std::to_string(players_.size()));
  std::vector<Keyframe> ks(count);
  std::vector<std::string> errs(count);
  // Runs on worker threads too: nothing may escape it.
  const std::function<void(uint32_t, uint32_t)> parse_range = [&](uint32_t b, uint32_t e) {
    for (uint32_t i = b; i < e; ++i) {
      if (!json[i]) {
        errs[i] = "null keyframe";
        continue;
      }
      try {
        Json doc;
        JsonParser jp{json[i], json[i] + length[i], {}};
        if (!jp.parse(doc)) {
          errs[i] = "bad JSON: " + jp.err;
          continue;
        }
        const Json* obj = doc.get("keyframe");
        if (!obj) {
          errs[i] = "no \"keyframe\" member";
          continue;
        }
        parse_keyframe(*obj, ks[i], errs[i]);
      } catch (const std::exception& ex) {
        errs[i] = std::string("parse failed: ") + ex.what();
      }
    }
  };
  // Parsing costs about a microsecond per small keyframe: batches of a few
  // hundred keyframes and more are split over the worker threads.
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  if (count >= 256 && hw > 1) {
    shared_pool().run(count, 32, parse_range);
  } else {
    parse_range(0, count);
  }
  for (uint32_t i = 0; i < count; ++i)
    if (!errs[i].empty())
      return fail(GBR_ERROR_INVALID_ARGUMENT,
                  "setEnvironmentKeyframes: environment " + std::to_string(first + i) + ": " + errs[i]);
  const std::string prefix = sensor_prefix ? sensor_prefix : "";
  for (uint32_t i = 0; i < count; ++i) {
    if (gbr_status s = players_[first + i]->set_single_keyframe(std::move(ks[i]))) return s;
    if (sensor_prefix)
      if (gbr_status s = set_sensor_from_keyframe(first + i, prefix)) return s;
  }
  return GBR_OK;
}

gbr_status ReplayRenderer::set_sensor_transform(uint32_t env, const float m[16]) {
  if (gbr_status s = check_env(env, "setSensorTransform")) return s;
  float view[16];
  if (!invert4(m, view)) return fail(GBR_ERROR_INVALID_ARGUMENT, "setSensorTransform: singular transform");
  std::memcpy(camera_[env].data(), m, 16 * sizeof(float));
  return renderer_->update_camera(env, projection_, view);
}

gbr_status ReplayRenderer::set_sensor_from_keyframe(uint32_t env, const std::string& prefix) {
  if (gbr_status s = check_env(env, "setSensorTransformsFromKeyframe")) return s;
  Player& p = *players_[env];
  if (p.keyframe_count() != 1)
    return fail(GBR_ERROR_STATE, "setSensorTransformsFromKeyframe: for environment " + std::to_string(env) +
                                     ", you have not yet called setEnvironmentKeyframe.");
  const std::string name = prefix + sensor_name_;
  const Transform* t = p.user_transform(name);
  if (!t)
    return fail(GBR_ERROR_NOT_FOUND, "setSensorTransformsFromKeyframe: couldn't find user transform \"" +
                                         name + "\" for environment " + std::to_string(env) + ".");
  float m[16];
  rigid_matrix(t->rotation, t->translation, m);
  return set_sensor_transform(env, m);
}

gbr_status ReplayRenderer::render(void* stream, uint32_t nc, void* const* color, uint64_t crow, uint32_t nd,
                                  void* const* depth, uint64_t drow) {
  TraceRange trace_("replay.render");
  if (!renderer_) return fail(GBR_ERROR_STATE, "render: the replay renderer is closed");
  const uint32_t n = env_count();
  if (nc && nc != n)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "ReplayRenderer::render(): expected " + std::to_string(n) +
                                                " color image views but got " + std::to_string(nc));
  if (nd && nd != n)
    return fail(GBR_ERROR_INVALID_ARGUMENT, "ReplayRenderer::render(): expected " + std::to_string(n) +
                                                " depth image views but got " + std::to_string(nd));
  for (uint32_t i = 0; i < nc; ++i)
    if (!color[i]) return fail(GBR_ERROR_INVALID_ARGUMENT, "render: null color destination");
  for (uint32_t i = 0; i < nd; ++i)
    if (!depth[i]) return fail(GBR_ERROR_INVALID_ARGUMENT, "render: null depth destination");
  const uint32_t mode = cfg_.draw_mode;
  if (gbr_status s = renderer_->draw(static_cast<cudaStream_t>(stream), mode, mode == GBR_DRAW_BATCHED))
    return s;
  if (cfg_.enable_hbao) {  // the classic replay renderer's HBAO (ClassicReplayRenderer.cpp:142, 326)
    gbr_hbao_config hc;
    gbr_hbao_config_init(&hc);
    if (gbr_status s = renderer_->hbao(hc, static_cast<cudaStream_t>(stream))) return s;
  }
  const int32_t w = cfg_.resolution[1], h = cfg_.resolution[0];
  // Destinations that are one packed array (environment i at base + i
  // images, rows without padding) take one gather and one copy per plane.
  auto packed = [&](void* const* d, uint32_t count, uint64_t row, size_t elem) {
    if (!count || row != uint64_t(w) * elem) return false;
    const size_t image = size_t(h) * row;
    for (uint32_t i = 1; i < count; ++i)
      if (static_cast<char*>(d[i]) != static_cast<char*>(d[0]) + i * image) return false;
    return true;
  };
  const bool pc = packed(color, nc, crow, 4), pd = packed(depth, nd, drow, 4);
  if (pc)
    if (gbr_status s = renderer_->scenes_into_async(GBR_PLANE_COLOR, 0, n, color[0])) return s;
  if (pd)
    if (gbr_status s = renderer_->scenes_into_async(GBR_PLANE_LINEAR_DEPTH, 0, n, depth[0])) return s;
  for (uint32_t i = 0; i < n && (!pc || !pd); ++i) {
    const int32_t x0 = int32_t(i % uint32_t(grid_[0])) * w, y0 = int32_t(i / uint32_t(grid_[0])) * h;
    const int32_t rect[4] = {x0, y0, x0 + w, y0 + h};
    if (nc && !pc)
      if (gbr_status s = renderer_->image_into_async(GBR_PLANE_COLOR, rect, color[i], crow)) return s;
    if (nd && !pd)
      if (gbr_status s = renderer_->image_into_async(GBR_PLANE_LINEAR_DEPTH, rect, depth[i], drow)) return s;
  }
  return renderer_->readback_wait();
}

gbr_status ReplayRenderer::unproject(uint32_t env, int32_t x, int32_t y, float origin[3], float dir[3]) const {
  if (gbr_status s = check_env(env, "unproject")) return s;
  const float w = float(cfg_.resolution[1]), h = float(cfg_.resolution[0]);
  const float vx = float(x), vy = float(cfg_.resolution[0] - y - 1);
  const float ndc[4] = {2.0f * vx / w - 1.0f, 2.0f * vy / h - 1.0f, 1.0f, 1.0f};
  float ip[16];
  if (!invert4(projection_, ip)) return fail(GBR_ERROR_STATE, "unproject: singular projection");
  const float* cam = camera_[env].data();
  float e[4], p[4];
  for (int r = 0; r < 4; ++r) e[r] = ip[r] * ndc[0] + ip[4 + r] * ndc[1] + ip[8 + r] * ndc[2] + ip[12 + r] * ndc[3];
  for (int r = 0; r < 4; ++r) p[r] = cam[r] * e[0] + cam[4 + r] * e[1] + cam[8 + r] * e[2] + cam[12 + r] * e[3];
  for (int i = 0; i < 3; ++i) origin[i] = cam[12 + i];
  float d[3] = {p[0] / p[3] - origin[0], p[1] / p[3] - origin[1], p[2] / p[3] - origin[2]};
  normalize3(d);
  std::memcpy(dir, d, sizeof d);
  return GBR_OK;
}

}  // namespace replay
}  // namespace gbr

// ------------------------------------------------------------------- C ABI
using gbr::replay::ReplayRenderer;

namespace {

ReplayRenderer* RR(gbr_replay* r) { return reinterpret_cast<ReplayRenderer*>(r); }

template <class F>
gbr_status guarded(gbr_replay* r, F&& f) {
  if (!r) {
    gbr::set_last_error("null replay renderer handle");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  try {
    gbr::set_last_error("");
    return f(*RR(r));
  } catch (const std::bad_alloc&) {
    gbr::set_last_error("host allocation failed");
    return GBR_ERROR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    gbr::set_last_error(e.what());
    return GBR_ERROR_STATE;
  }
}

gbr_status null_arg(const char* what) {
  gbr::set_last_error(std::string("null argument: ") + what);
  return GBR_ERROR_INVALID_ARGUMENT;
}

}  // namespace

#define GBR_ARG(p) \
  if (!(p)) return null_arg(#p)

extern "C" {

void gbr_replay_config_init(gbr_replay_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->num_environments = 1;
  c->standalone = 1;
  c->enable_frustum_culling = 1;
  c->resolution[0] = c->resolution[1] = 128;
  c->hfov_degrees = 90.0f;
  c->near_plane = 0.01f;
  c->far_plane = 1000.0f;
  c->ortho_scale = 0.1f;
  c->ambient_factor = 0.1f;
  c->draw_mode = GBR_DRAW_BATCHED;
}

gbr_status gbr_replay_create(const gbr_replay_config* config, gbr_replay** out) {
  GBR_ARG(config);
  GBR_ARG(out);
  try {
    gbr::set_last_error("");
    gbr_status st;
    *out = reinterpret_cast<gbr_replay*>(ReplayRenderer::create(*config, st));
    return st;
  } catch (const std::bad_alloc&) {
    gbr::set_last_error("host allocation failed");
    return GBR_ERROR_OUT_OF_MEMORY;
  }
}

void gbr_replay_destroy(gbr_replay* r) { delete RR(r); }

gbr_status gbr_replay_close(gbr_replay* r) {
  return guarded(r, [](ReplayRenderer& rr) { return rr.close(); });
}

gbr_status gbr_replay_renderer(gbr_replay* r, gbr_renderer** out) {
  GBR_ARG(out);
  return guarded(r, [&](ReplayRenderer& rr) {
    if (rr.closed()) {
      gbr::set_last_error("the replay renderer is closed");
      return GBR_ERROR_STATE;
    }
    *out = reinterpret_cast<gbr_renderer*>(rr.renderer());
    return GBR_OK;
  });
}

gbr_status gbr_replay_environment_grid_size(int32_t n, int32_t out[2]) {
  GBR_ARG(out);
  if (n <= 0) {
    gbr::set_last_error("environmentGridSize: count must be positive");
    return GBR_ERROR_INVALID_ARGUMENT;
  }
  const int32_t x = int32_t(std::ceil(std::sqrt(float(n))));
  out[0] = x;
  out[1] = (n + x - 1) / x;
  return GBR_OK;
}

gbr_status gbr_replay_preload_file(gbr_replay* r, const char* filename) {
  GBR_ARG(filename);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.preload_file(filename); });
}

gbr_status gbr_replay_environment_count(gbr_replay* r, uint32_t* out) {
  GBR_ARG(out);
  return guarded(r, [&](ReplayRenderer& rr) {
    *out = rr.env_count();
    return GBR_OK;
  });
}

gbr_status gbr_replay_sensor_size(gbr_replay* r, uint32_t env, int32_t out[2]) {
  GBR_ARG(out);
  return guarded(r, [&](ReplayRenderer& rr) {
    if (gbr_status s = rr.check_env(env, "sensorSize")) return s;
    out[0] = rr.config().resolution[1];
    out[1] = rr.config().resolution[0];
    return GBR_OK;
  });
}

gbr_status gbr_replay_clear_environment(gbr_replay* r, uint32_t env) {
  return guarded(r, [&](ReplayRenderer& rr) { return rr.clear_environment(env); });
}

gbr_status gbr_replay_set_environment_keyframe(gbr_replay* r, uint32_t env, const char* json, uint64_t length) {
  GBR_ARG(json);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.set_keyframe_json(env, json, length, true); });
}

gbr_status gbr_replay_set_environment_keyframe_unwrapped(gbr_replay* r, uint32_t env, const char* json,
                                                         uint64_t length) {
  GBR_ARG(json);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.set_keyframe_json(env, json, length, false); });
}

gbr_status gbr_replay_set_environment_keyframes(gbr_replay* r, uint32_t first_env, uint32_t count,
                                                const char* const* json, const uint64_t* length,
                                                const char* sensor_prefix) {
  if (count) {
    GBR_ARG(json);
    GBR_ARG(length);
  }
  return guarded(r, [&](ReplayRenderer& rr) {
    return rr.set_keyframe_batch(first_env, count, json, length, sensor_prefix);
  });
}

gbr_status gbr_replay_set_keyframes(gbr_replay* r, uint32_t env, const char* json, uint64_t length) {
  GBR_ARG(json);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.set_keyframes_json(env, json, length); });
}

gbr_status gbr_replay_set_keyframe_index(gbr_replay* r, uint32_t env, int32_t index) {
  return guarded(r, [&](ReplayRenderer& rr) {
    if (gbr_status s = rr.check_env(env, "setKeyframeIndex")) return s;
    return rr.player(env).set_keyframe_index(index);
  });
}

gbr_status gbr_replay_keyframe_count(gbr_replay* r, uint32_t env, int32_t* count, int32_t* index) {
  GBR_ARG(count);
  GBR_ARG(index);
  return guarded(r, [&](ReplayRenderer& rr) {
    if (gbr_status s = rr.check_env(env, "getNumKeyframes")) return s;
    *count = rr.player(env).keyframe_count();
    *index = rr.player(env).keyframe_index();
    return GBR_OK;
  });
}

gbr_status gbr_replay_user_transform(gbr_replay* r, uint32_t env, const char* name, float translation[3],
                                     float rotation[4], int32_t* found) {
  GBR_ARG(name);
  GBR_ARG(translation);
  GBR_ARG(rotation);
  GBR_ARG(found);
  return guarded(r, [&](ReplayRenderer& rr) {
    if (gbr_status s = rr.check_env(env, "getUserTransform")) return s;
    const gbr::replay::Transform* t = rr.player(env).user_transform(name);
    *found = t ? 1 : 0;
    if (t) {
      std::memcpy(translation, t->translation, 3 * sizeof(float));
      rotation[0] = t->rotation.x;
      rotation[1] = t->rotation.y;
      rotation[2] = t->rotation.z;
      rotation[3] = t->rotation.w;
    }
    return GBR_OK;
  });
}

gbr_status gbr_replay_set_sensor_transform(gbr_replay* r, uint32_t env, const char* sensor_name,
                                           const float transform[16]) {
  (void)sensor_name;
  GBR_ARG(transform);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.set_sensor_transform(env, transform); });
}

gbr_status gbr_replay_set_sensor_transforms_from_keyframe(gbr_replay* r, uint32_t env, const char* prefix) {
  GBR_ARG(prefix);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.set_sensor_from_keyframe(env, prefix); });
}

gbr_status gbr_replay_render(gbr_replay* r, void* stream, uint32_t color_count, void* const* color,
                             uint64_t color_row_bytes, uint32_t depth_count, void* const* depth,
                             uint64_t depth_row_bytes) {
  if (color_count) GBR_ARG(color);
  if (depth_count) GBR_ARG(depth);
  return guarded(r, [&](ReplayRenderer& rr) {
    return rr.render(stream, color_count, color, color_row_bytes, depth_count, depth, depth_row_bytes);
  });
}

gbr_status gbr_replay_unproject(gbr_replay* r, uint32_t env, int32_t x, int32_t y, float origin[3],
                                float direction[3]) {
  GBR_ARG(origin);
  GBR_ARG(direction);
  return guarded(r, [&](ReplayRenderer& rr) { return rr.unproject(env, x, y, origin, direction); });
}

}  // extern "C"
