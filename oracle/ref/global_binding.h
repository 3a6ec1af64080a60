// global_binding.h -- stand-in for shaders/src/hala-pathtracer/inc/global.glsl
// when the reference's shaders are compiled as host code (oracle/_ref).
//
// global.glsl only declares the descriptor-set layout; here the same names
// are host objects bound by the harness (ref_harness.inl). MainUBO keeps the
// field names and order of inc/global.glsl:11-30; it is per thread because
// the harness renders different frames on different threads.
#pragma once

extern accelerationStructureEXT g_tlas;
extern image2D g_final_image;
extern image2D g_accum_image;
extern image2D g_albedo_image;
extern image2D g_normal_image;
extern texture2D g_blue_noise;
extern sampler2D g_env_map;
extern texture2D g_env_map_dist[2];
extern sampler g_env_map_dist_sampler;

struct MainUBO {
  vec4 ground_color;
  vec4 sky_color;
  vec2 resolution;
  uint max_depth;
  uint rr_depth;
  uint frame_index;
  uint camera_index;
  uint env_type;
  uint env_map_width;
  uint env_map_height;
  float env_total_sum;
  float env_rotation;
  float env_intensity;
  float exposure_value;
  bool enable_tonemap;
  bool enable_aces;
  bool use_simple_aces;
  uint num_of_lights;
};
extern thread_local MainUBO g_main_ubo_inst;

struct CamerasBuffer {
  Camera cameras[MAX_CAMERAS];
};
extern CamerasBuffer g_cameras_buf_inst;

struct LightsBuffer {
  Light lights[MAX_LIGHTS];
};
extern LightsBuffer g_lights_buf_inst;

struct MaterialBuffer {
  Material data;
};
extern MaterialBuffer* g_materials;

struct PrimitivesBuffer {
  Primitive data;
};
extern PrimitivesBuffer* g_primitives;

extern sampler2D* g_textures;
