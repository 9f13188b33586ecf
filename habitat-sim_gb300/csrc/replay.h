// Batch replay renderer: gfx-replay keyframes -> batch renderer calls.
//
// Host-side driver around Renderer, restating habitat-sim's
// esp::sim::BatchReplayRenderer (src/esp/sim/BatchReplayRenderer.cpp),
// esp::gfx::replay::Player (src/esp/gfx/replay/Player.cpp) and
// esp::sim::BatchPlayerImplementation (src/esp/sim/BatchPlayerImplementation.cpp).
#pragma once
#include <array>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gbr_replay.h"
#include "json.h"
#include "pool.h"

namespace gbr {

class Renderer;

namespace replay {

struct Quat {
  float x = 0, y = 0, z = 0, w = 1;
};

// gfx/replay/Keyframe.h:20-27.
struct Transform {
  float translation[3] = {0, 0, 0};
  Quat rotation;
};

// assets::AssetInfo (the fields the batch player reads: the file and its
// coordinate frame, io/JsonEspTypes.cpp:220-232).
struct AssetInfo {
  int type = 0;
  std::string filepath;
  float up[3] = {0, 1, 0};
  float front[3] = {0, 0, -1};
  float origin[3] = {0, 0, 0};
};

// assets::RenderAssetInstanceCreationInfo (io/JsonEspTypes.h:91-118).
struct Creation {
  std::string filepath;
  bool has_scale = false;
  float scale[3] = {1, 1, 1};
  uint32_t flags = 0;  // 1 static, 2 RGBD, 4 semantic, 8 texture-based semantic
  std::string light_setup_key;
  int rig_id = -1;
};

struct Metadata {
  int object_id = -1;
  int semantic_id = -1;
};

// gfx::LightInfo: vector (w = 0 directional, 1 point), colour, position model.
struct Light {
  float vector[4] = {0, 0, 0, 0};
  float color[3] = {1, 1, 1};
  bool global = true;
};

// gfx/replay/Keyframe.h:70-91.
struct Keyframe {
  std::vector<AssetInfo> loads;
  std::vector<std::pair<int, Creation>> creations;
  std::vector<int> deletions;
  std::vector<std::pair<int, Metadata>> metadata;
  std::vector<std::pair<int, Transform>> state_updates;
  std::map<std::string, Transform> user_transforms;
  std::vector<Light> lights;
  bool lights_changed = false;
};

// Keyframe JSON (io/JsonEspTypes.cpp:102-201).  Returns false with a message.
bool parse_keyframe(const Json& obj, Keyframe& out, std::string& err);

// Rotation matrix of a unit quaternion, column-major 3x3.
void quat_to_matrix(const Quat& q, float m[9]);
// Rotation taking unit vector a to unit vector b.
Quat quat_between(const float a[3], const float b[3]);
Quat quat_mul(const Quat& a, const Quat& b);
Quat quat_normalized(const Quat& q);
void quat_rotate(const Quat& q, const float v[3], float out[3]);
// Frame-to-world rotation of a coordinate frame (geo/CoordinateFrame.cpp:31-43).
Quat frame_to_world(const float up[3], const float front[3]);
// Rigid transform [R(q) | t], column-major 4x4.
void rigid_matrix(const Quat& q, const float t[3], float m[16]);
// General 4x4 inverse (cofactor expansion); false if singular.
bool invert4(const float m[16], float out[16]);
// Projection of the sensor (sensor/CameraSensor.cpp:44-60).
void sensor_projection(const gbr_replay_config& c, float p[16]);

// BatchPlayerImplementation: one environment = one renderer scene.  Node
// handles are the hierarchy's root node index + 1 (0 = failed creation).
class BatchPlayer {
 public:
  BatchPlayer(Renderer& r, uint32_t scene, bool quiet) : r_(r), scene_(scene), quiet_(quiet) {}
  gbr_status load_and_create(const AssetInfo& info, const Creation& c, uint64_t* node);
  gbr_status delete_all();
  gbr_status set_transform(uint64_t node, const Transform& t);
  gbr_status set_matrix(uint64_t node, const float m[16]);
  gbr_status get_matrix(uint64_t node, float m[16]) const;
  gbr_status set_metadata(uint64_t node, const Metadata& md);
  gbr_status change_lights(const std::vector<Light>& lights);
  void warn(const std::string& msg) const;

 private:
  Renderer& r_;
  uint32_t scene_;
  bool quiet_;
};

// Player (gfx/replay/Player.cpp): keyframes of one environment and the
// instances created from them.
class Player {
 public:
  explicit Player(BatchPlayer impl) : impl_(std::move(impl)) {}
  void set_keyframes(std::vector<Keyframe> k);
  gbr_status set_single_keyframe(Keyframe k);
  gbr_status set_keyframe_index(int index);
  int keyframe_count() const { return int(keyframes_.size()); }
  int keyframe_index() const { return index_; }
  const Transform* user_transform(const std::string& name) const;
  gbr_status close();

 private:
  struct Record {
    Creation creation;
    Metadata metadata;
  };
  gbr_status clear_frame();
  gbr_status apply(const Keyframe& k);
  gbr_status process_deletions(const Keyframe& k);

  BatchPlayer impl_;
  std::vector<Keyframe> keyframes_;
  int index_ = -1;
  std::unordered_map<std::string, AssetInfo> asset_infos_;
  std::set<std::string> failed_;
  std::map<int, uint64_t> created_;  // instance key -> node handle, in key order
  std::map<int, Record> records_;
};

class ReplayRenderer {
 public:
  static ReplayRenderer* create(const gbr_replay_config& cfg, gbr_status& st);
  ~ReplayRenderer();
  gbr_status close();
  bool closed() const { return renderer_ == nullptr; }
  Renderer* renderer() const { return renderer_; }
  uint32_t env_count() const { return uint32_t(players_.size()); }
  const gbr_replay_config& config() const { return cfg_; }

  gbr_status check_env(uint32_t env, const char* fn) const;
  gbr_status preload_file(const char* filename);
  gbr_status clear_environment(uint32_t env);
  gbr_status set_keyframe_json(uint32_t env, const char* json, uint64_t n, bool wrapped);
  gbr_status set_keyframes_json(uint32_t env, const char* json, uint64_t n);
  gbr_status set_keyframe_batch(uint32_t first, uint32_t count, const char* const* json,
                                const uint64_t* length, const char* sensor_prefix);
  Player& player(uint32_t env) { return *players_[env]; }
  gbr_status set_sensor_transform(uint32_t env, const float m[16]);
  gbr_status set_sensor_from_keyframe(uint32_t env, const std::string& prefix);
  gbr_status render(void* stream, uint32_t nc, void* const* color, uint64_t crow, uint32_t nd,
                    void* const* depth, uint64_t drow);
  gbr_status unproject(uint32_t env, int32_t x, int32_t y, float origin[3], float dir[3]) const;

 private:
  ReplayRenderer() = default;
  gbr_replay_config cfg_{};
  std::string sensor_name_;
  float projection_[16] = {};
  int32_t grid_[2] = {1, 1};
  Renderer* renderer_ = nullptr;
  std::vector<std::unique_ptr<Player>> players_;
  std::vector<std::array<float, 16>> camera_;  // camera-to-world per environment
};

}  // namespace replay
}  // namespace gbr
