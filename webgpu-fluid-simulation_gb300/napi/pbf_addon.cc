// pbf_addon.cc - Node-API addon over the C ABI of libpbf_gb300.
//
// It gives a TypeScript host the calls of the reference's simulator and
// renderer classes (src/simulator/SPH.ts, src/simulator/PBF/PBFConfig.ts,
// src/simulator/PBF/PBF.ts, src/renderer/filteredParticleFluid/fluid.ts);
// pbf.ts wraps them back into classes with the reference's method names.
// Every export takes plain JS values (numbers, arrays, typed arrays, strings,
// plain objects) and the handle created by `create` / `rendererCreate`.
// A failing library call throws an Error whose `code` is the pbf_status name
// and whose message carries pbf_last_error, where the reference throws
// (PBFConfig.ts:50-55, volumeMap.ts:31-33); a wrong argument type throws a
// TypeError before the library is called.
#include <node_api.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "pbf_gb300.h"

namespace {

// ---------------------------------------------------------------- handles

// The simulator handle behind a JS External.  `pending` pins the typed array
// of an asynchronous position read until `synchronize`, so the garbage
// collector cannot free the memory the copy stream is writing.
struct Sim {
  pbf_handle* h = nullptr;
  napi_ref pending = nullptr;
};

struct Renderer {
  pbf_renderer* r = nullptr;
};

constexpr uint32_t kSimTag = 0x50424653u;  // tags the External's payload type
constexpr uint32_t kRenTag = 0x50424652u;
struct Boxed {
  uint32_t tag;
  Sim sim;
  Renderer ren;
};

const char* status_name(int rc) {
  switch (rc) {
    case PBF_EINVAL: return "PBF_EINVAL";
    case PBF_ECAPACITY: return "PBF_ECAPACITY";
    case PBF_EFORMAT: return "PBF_EFORMAT";
    case PBF_ECUDA: return "PBF_ECUDA";
    case PBF_ETIMEOUT: return "PBF_ETIMEOUT";
    case PBF_EDIVERGED: return "PBF_EDIVERGED";
    case PBF_ESTATE: return "PBF_ESTATE";
    default: return "PBF_ERROR";
  }
}

// Throws a JS Error for a failed library call; returns nullptr (undefined).
napi_value fail(napi_env env, const pbf_handle* h, int rc, const char* what) {
  std::string msg = std::string(what) + " failed: ";
  const char* detail = h ? pbf_last_error(h) : nullptr;
  msg += (detail && *detail) ? detail : status_name(rc);
  napi_throw_error(env, status_name(rc), msg.c_str());
  return nullptr;
}

napi_value type_error(napi_env env, const char* msg) {
  napi_throw_type_error(env, "ERR_INVALID_ARG_TYPE", msg);
  return nullptr;
}

napi_value undefined(napi_env env) {
  napi_value v = nullptr;
  napi_get_undefined(env, &v);
  return v;
}

napi_value number(napi_env env, double x) {
  napi_value v = nullptr;
  napi_create_double(env, x, &v);
  return v;
}

napi_value boolean(napi_env env, bool b) {
  napi_value v = nullptr;
  napi_get_boolean(env, b, &v);
  return v;
}

// Up to `max` arguments; missing ones read as undefined.
struct Args {
  napi_value v[6];
  size_t n = 6;
  bool ok;
  Args(napi_env env, napi_callback_info info) {
    ok = napi_get_cb_info(env, info, &n, v, nullptr, nullptr) == napi_ok;
    napi_value u = undefined(env);
    for (size_t i = n; i < 6; ++i) v[i] = u;
  }
};

void finalize_boxed(napi_env, void* data, void*) {
  Boxed* b = static_cast<Boxed*>(data);
  if (b->tag == kSimTag && b->sim.h) pbf_destroy(b->sim.h);
  if (b->tag == kRenTag && b->ren.r) pbf_renderer_destroy(b->ren.r);
  delete b;
}

Boxed* unbox(napi_env env, napi_value v, uint32_t tag) {
  napi_valuetype t;
  if (napi_typeof(env, v, &t) != napi_ok || t != napi_external) return nullptr;
  void* p = nullptr;
  if (napi_get_value_external(env, v, &p) != napi_ok || !p) return nullptr;
  Boxed* b = static_cast<Boxed*>(p);
  return b->tag == tag ? b : nullptr;
}

// The live simulator of argument 0, or nullptr after throwing.
Sim* sim_arg(napi_env env, napi_value v) {
  Boxed* b = unbox(env, v, kSimTag);
  if (!b) {
    type_error(env, "argument 0 must be a simulator handle from create()");
    return nullptr;
  }
  if (!b->sim.h) {
    napi_throw_error(env, "PBF_ESTATE", "the simulator handle was destroyed");
    return nullptr;
  }
  return &b->sim;
}

Renderer* renderer_arg(napi_env env, napi_value v) {
  Boxed* b = unbox(env, v, kRenTag);
  if (!b) {
    type_error(env, "argument 0 must be a renderer handle from rendererCreate()");
    return nullptr;
  }
  if (!b->ren.r) {
    napi_throw_error(env, "PBF_ESTATE", "the renderer handle was destroyed");
    return nullptr;
  }
  return &b->ren;
}

// ---------------------------------------------------------------- values

bool is_type(napi_env env, napi_value v, napi_valuetype want) {
  napi_valuetype t;
  return napi_typeof(env, v, &t) == napi_ok && t == want;
}

bool get_number(napi_env env, napi_value v, double* out) {
  return is_type(env, v, napi_number) && napi_get_value_double(env, v, out) == napi_ok;
}

bool get_u32(napi_env env, napi_value v, uint32_t* out) {
  double d;
  if (!get_number(env, v, &d) || !(d >= 0.0) || d > 4294967295.0 || d != std::floor(d)) return false;
  *out = static_cast<uint32_t>(d);
  return true;
}

// n numbers from a JS array or a Float32Array / Float64Array (three.js
// Vector3 components or Matrix4.elements).
bool get_numbers(napi_env env, napi_value v, double* out, size_t n) {
  bool ta = false, arr = false;
  napi_is_typedarray(env, v, &ta);
  if (ta) {
    napi_typedarray_type t;
    size_t len = 0, off = 0;
    void* data = nullptr;
    napi_value ab;
    if (napi_get_typedarray_info(env, v, &t, &len, &data, &ab, &off) != napi_ok || len != n) return false;
    if (t == napi_float32_array) {
      for (size_t i = 0; i < n; ++i) out[i] = static_cast<const float*>(data)[i];
      return true;
    }
    if (t == napi_float64_array) {
      for (size_t i = 0; i < n; ++i) out[i] = static_cast<const double*>(data)[i];
      return true;
    }
    return false;
  }
  napi_is_array(env, v, &arr);
  if (!arr) return false;
  uint32_t len = 0;
  if (napi_get_array_length(env, v, &len) != napi_ok || len != n) return false;
  for (uint32_t i = 0; i < len; ++i) {
    napi_value e;
    if (napi_get_element(env, v, i, &e) != napi_ok || !get_number(env, e, &out[i])) return false;
  }
  return true;
}

bool get_floats(napi_env env, napi_value v, float* out, size_t n) {
  double tmp[16];
  if (n > 16 || !get_numbers(env, v, tmp, n)) return false;
  for (size_t i = 0; i < n; ++i) out[i] = static_cast<float>(tmp[i]);
  return true;
}

// A typed array's storage when its element type is `want`.
bool get_typed(napi_env env, napi_value v, napi_typedarray_type want, void** data, size_t* length) {
  bool ta = false;
  if (napi_is_typedarray(env, v, &ta) != napi_ok || !ta) return false;
  napi_typedarray_type t;
  size_t off = 0;
  napi_value ab;
  return napi_get_typedarray_info(env, v, &t, length, data, &ab, &off) == napi_ok && t == want;
}

// obj[name] when present and not undefined.
bool property(napi_env env, napi_value obj, const char* name, napi_value* out) {
  bool has = false;
  if (napi_has_named_property(env, obj, name, &has) != napi_ok || !has) return false;
  if (napi_get_named_property(env, obj, name, out) != napi_ok) return false;
  return !is_type(env, *out, napi_undefined);
}

// Optional numeric member: absent keeps *out; present but not a number fails.
bool opt_number(napi_env env, napi_value obj, const char* name, float* out) {
  napi_value v;
  if (!property(env, obj, name, &v)) return true;
  double d;
  if (!get_number(env, v, &d)) return false;
  *out = static_cast<float>(d);
  return true;
}

bool opt_u32(napi_env env, napi_value obj, const char* name, uint32_t* out) {
  napi_value v;
  if (!property(env, obj, name, &v)) return true;
  return get_u32(env, v, out);
}

bool opt_vec3(napi_env env, napi_value obj, const char* name, float out[3]) {
  napi_value v;
  if (!property(env, obj, name, &v)) return true;
  return get_floats(env, v, out, 3);
}

void set_number(napi_env env, napi_value obj, const char* name, double x) {
  napi_set_named_property(env, obj, name, number(env, x));
}

// ---------------------------------------------------------------- simulator

// create(config?) -> handle.  `new PBF()` + `initResource()` (PBF.ts:67-69,
// 262-279; PBFConfig.ts:19-29: r = 0.006, one substep).  Optional members:
// particleRadius, kernelRadius, restDensity, timeStep, stepCount,
// maxParticles, maxNeighbors, domainMin, domainMax, fastMath.
napi_value Create(napi_env env, napi_callback_info info) {
  Args a(env, info);
  pbf_config c;
  pbf_config_default(&c);
  if (!is_type(env, a.v[0], napi_undefined)) {
    if (!is_type(env, a.v[0], napi_object)) return type_error(env, "create(config): config must be an object");
    bool fast = c.fp_mode == PBF_FP_FAST;
    napi_value fv;
    if (property(env, a.v[0], "fastMath", &fv)) {
      if (!is_type(env, fv, napi_boolean) || napi_get_value_bool(env, fv, &fast) != napi_ok)
        return type_error(env, "create(config): fastMath must be a boolean");
    }
    c.fp_mode = fast ? PBF_FP_FAST : PBF_FP_EXACT;
    if (!opt_number(env, a.v[0], "particleRadius", &c.particle_radius) ||
        !opt_number(env, a.v[0], "kernelRadius", &c.kernel_radius) ||
        !opt_number(env, a.v[0], "restDensity", &c.rest_density) ||
        !opt_number(env, a.v[0], "timeStep", &c.time_step) || !opt_u32(env, a.v[0], "stepCount", &c.substeps) ||
        !opt_u32(env, a.v[0], "maxParticles", &c.max_particles) ||
        !opt_u32(env, a.v[0], "maxNeighbors", &c.max_neighbors) ||
        !opt_vec3(env, a.v[0], "domainMin", c.domain_min) || !opt_vec3(env, a.v[0], "domainMax", c.domain_max))
      return type_error(env, "create(config): numeric members must be numbers, domainMin/domainMax 3 numbers");
  }
  pbf_handle* h = nullptr;
  const int rc = pbf_create(&c, &h);
  if (rc) return fail(env, nullptr, rc, "create");
  Boxed* b = new Boxed{kSimTag, Sim{h, nullptr}, Renderer{}};
  napi_value ext;
  if (napi_create_external(env, b, finalize_boxed, nullptr, &ext) != napi_ok) {
    pbf_destroy(h);
    delete b;
    napi_throw_error(env, nullptr, "create: napi_create_external failed");
    return nullptr;
  }
  return ext;
}

// destroy(h): frees the device state now instead of at garbage collection.
napi_value Destroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  pbf_destroy(s->h);
  s->h = nullptr;
  if (s->pending) {
    napi_delete_reference(env, s->pending);
    s->pending = nullptr;
  }
  return undefined(env);
}

// reset(h): PBF.reset (PBF.ts:71-89).
napi_value Reset(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  const int rc = pbf_reset(s->h);
  return rc ? fail(env, s->h, rc, "reset") : undefined(env);
}

// setConfig(h, {iteration, XSPH, vorticity, surfaceTension, gravity}):
// PBFConfig.setConfig (PBFConfig.ts:31-46); all five members are required.
napi_value SetConfig(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  if (!is_type(env, a.v[1], napi_object)) return type_error(env, "setConfig(h, config): config must be an object");
  static const char* kNames[5] = {"iteration", "XSPH", "vorticity", "surfaceTension", "gravity"};
  double x[5];
  for (int i = 0; i < 5; ++i) {
    napi_value v;
    if (!property(env, a.v[1], kNames[i], &v) || !get_number(env, v, &x[i]))
      return type_error(env, (std::string("setConfig: member '") + kNames[i] + "' must be a number").c_str());
  }
  if (!(x[0] >= 0.0) || x[0] > 1000.0 || x[0] != std::floor(x[0]))
    return type_error(env, "setConfig: 'iteration' must be a whole number of iterations");
  pbf_options o;
  o.iterations = static_cast<uint32_t>(x[0]);
  o.xsph = static_cast<float>(x[1]);
  o.vorticity = static_cast<float>(x[2]);
  o.surface_tension = static_cast<float>(x[3]);
  o.gravity = static_cast<float>(x[4]);
  const int rc = pbf_set_options(s->h, &o);
  return rc ? fail(env, s->h, rc, "setConfig") : undefined(env);
}

// getConfig(h) -> {iteration, XSPH, vorticity, surfaceTension, gravity}.
napi_value GetConfig(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  pbf_options o;
  const int rc = pbf_get_options(s->h, &o);
  if (rc) return fail(env, s->h, rc, "getConfig");
  napi_value obj;
  napi_create_object(env, &obj);
  set_number(env, obj, "iteration", o.iterations);
  set_number(env, obj, "XSPH", o.xsph);
  set_number(env, obj, "vorticity", o.vorticity);
  set_number(env, obj, "surfaceTension", o.surface_tension);
  set_number(env, obj, "gravity", o.gravity);
  return obj;
}

// voxelizeCube(h, min[3], max[3]) -> points added (SPH.ts:99-121).
napi_value VoxelizeCube(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  float mn[3], mx[3];
  if (!get_floats(env, a.v[1], mn, 3) || !get_floats(env, a.v[2], mx, 3))
    return type_error(env, "voxelizeCube(h, min, max): min and max must be 3 numbers each");
  uint32_t added = 0;
  const int rc = pbf_voxelize_cube(s->h, mn, mx, &added);
  return rc ? fail(env, s->h, rc, "voxelizeCube") : number(env, added);
}

// voxelizeSphere(h, center[3], radius) -> points added (SPH.ts:123-149).
napi_value VoxelizeSphere(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  float c[3];
  double r;
  if (!get_floats(env, a.v[1], c, 3) || !get_number(env, a.v[2], &r))
    return type_error(env, "voxelizeSphere(h, center, radius): center must be 3 numbers, radius a number");
  uint32_t added = 0;
  const int rc = pbf_voxelize_sphere(s->h, c, static_cast<float>(r), &added);
  return rc ? fail(env, s->h, rc, "voxelizeSphere") : number(env, added);
}

// voxelizeMesh(h, Float32Array positions, Uint32Array|null index,
// matrixWorld[16]) -> points added (SPH.ts:151-187).  A null index takes
// the geometry as non-indexed: triangle i is vertices 3i, 3i+1, 3i+2.
napi_value VoxelizeMesh(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  void* pos = nullptr;
  size_t np = 0;
  if (!get_typed(env, a.v[1], napi_float32_array, &pos, &np) || np % 3 != 0)
    return type_error(env, "voxelizeMesh: positions must be a Float32Array of xyz triples");
  std::vector<uint32_t> own;
  const uint32_t* idx = nullptr;
  size_t ni = 0;
  if (is_type(env, a.v[2], napi_null) || is_type(env, a.v[2], napi_undefined)) {
    own.resize(np / 3);
    for (size_t i = 0; i < own.size(); ++i) own[i] = static_cast<uint32_t>(i);
    idx = own.data();
    ni = own.size();
  } else {
    void* p = nullptr;
    if (!get_typed(env, a.v[2], napi_uint32_array, &p, &ni))
      return type_error(env, "voxelizeMesh: index must be a Uint32Array or null");
    idx = static_cast<const uint32_t*>(p);
  }
  if (ni % 3 != 0) return type_error(env, "voxelizeMesh: the index length must be a multiple of 3");
  double world[16];
  if (!get_numbers(env, a.v[3], world, 16))
    return type_error(env, "voxelizeMesh: matrixWorld must be 16 numbers (Matrix4.elements)");
  uint32_t added = 0;
  const int rc = pbf_voxelize_mesh(s->h, static_cast<const float*>(pos), static_cast<uint32_t>(np / 3), idx,
                                   static_cast<uint32_t>(ni / 3), world, &added);
  return rc ? fail(env, s->h, rc, "voxelizeMesh") : number(env, added);
}

// setParticlePosition(h): PBFConfig.setParticlePosition (PBFConfig.ts:48-62).
napi_value SetParticlePosition(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  const int rc = pbf_set_particle_position(s->h);
  return rc ? fail(env, s->h, rc, "setParticlePosition") : undefined(env);
}

// setBoundaryData(h, text): PBF.setBoundaryData with the .cdm text (PBF.ts:91-94).
napi_value SetBoundaryData(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  if (!is_type(env, a.v[1], napi_string)) return type_error(env, "setBoundaryData(h, text): text must be a string");
  size_t len = 0;
  if (napi_get_value_string_utf8(env, a.v[1], nullptr, 0, &len) != napi_ok)
    return type_error(env, "setBoundaryData: unreadable string");
  std::string text(len + 1, '\0');
  napi_get_value_string_utf8(env, a.v[1], &text[0], text.size(), &len);
  const int rc = pbf_set_boundary_data(s->h, text.data(), len);
  return rc ? fail(env, s->h, rc, "setBoundaryData") : undefined(env);
}

// run(h): one substep (PBF.run, PBF.ts:398-448).
napi_value Run(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  const int rc = pbf_run(s->h);
  return rc ? fail(env, s->h, rc, "run") : undefined(env);
}

// step(h, frames): `frames` x stepCount substeps (src/controller.ts:375-376).
napi_value Step(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  uint32_t frames = 1;
  if (!is_type(env, a.v[1], napi_undefined) && !get_u32(env, a.v[1], &frames))
    return type_error(env, "step(h, frames): frames must be a whole number");
  const int rc = pbf_step(s->h, frames);
  return rc ? fail(env, s->h, rc, "step") : undefined(env);
}

// runTimestamp(h) -> [integrate, neighbour search, constraints, non-pressure] ms
// (PBF.runTimestamp, PBF.ts:450-510).
napi_value RunTimestamp(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  float ms[4];
  const int rc = pbf_run_timestamp(s->h, ms);
  if (rc) return fail(env, s->h, rc, "runTimestamp");
  napi_value arr;
  napi_create_array_with_length(env, 4, &arr);
  for (uint32_t i = 0; i < 4; ++i) napi_set_element(env, arr, i, number(env, ms[i]));
  return arr;
}

napi_value ParticleCount(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  return number(env, pbf_particle_count(s->h));
}

// setPaused(h, paused) / isPaused(h): SPH.pause (SPH.ts:29, 82-84).
napi_value SetPaused(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  bool p = false;
  if (!is_type(env, a.v[1], napi_boolean) || napi_get_value_bool(env, a.v[1], &p) != napi_ok)
    return type_error(env, "setPaused(h, paused): paused must be a boolean");
  const int rc = pbf_set_paused(s->h, p ? 1 : 0);
  return rc ? fail(env, s->h, rc, "setPaused") : undefined(env);
}

napi_value IsPaused(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  return boolean(env, pbf_is_paused(s->h) == 1);
}

// Float32Array of at least 4 n floats for the positions.
bool position_target(napi_env env, Sim* s, napi_value v, float** data, size_t* bytes) {
  void* p = nullptr;
  size_t len = 0;
  if (!get_typed(env, v, napi_float32_array, &p, &len)) return false;
  const size_t need = static_cast<size_t>(pbf_particle_count(s->h)) * 4;
  if (len < need) return false;
  *data = static_cast<float*>(p);
  *bytes = need * sizeof(float);
  return true;
}

// copyPositions(h, Float32Array): the `position` buffer (x, y, z, density by
// particle id, SPH.ts:39) read back now.
napi_value CopyPositions(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  float* data = nullptr;
  size_t bytes = 0;
  if (!position_target(env, s, a.v[1], &data, &bytes))
    return type_error(env, "copyPositions(h, out): out must be a Float32Array of 4 x particleCount floats");
  if (bytes == 0) return undefined(env);
  const int rc = pbf_copy_field(s->h, PBF_FIELD_POSITION, data, bytes);
  return rc ? fail(env, s->h, rc, "copyPositions") : undefined(env);
}

// copyPositionsAsync(h, Float32Array): the last frame's positions, written
// into `out` while the next frames run; complete after synchronize(h).
// The array is kept alive until then.
napi_value CopyPositionsAsync(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  float* data = nullptr;
  size_t bytes = 0;
  if (!position_target(env, s, a.v[1], &data, &bytes))
    return type_error(env, "copyPositionsAsync(h, out): out must be a Float32Array of 4 x particleCount floats");
  if (bytes == 0) return undefined(env);
  if (s->pending) {
    // an earlier read into another array: finish it before its array is released
    const int rc = pbf_synchronize(s->h);
    if (rc) return fail(env, s->h, rc, "copyPositionsAsync");
    napi_delete_reference(env, s->pending);
    s->pending = nullptr;
  }
  const int rc = pbf_copy_positions_async(s->h, data, bytes);
  if (rc) return fail(env, s->h, rc, "copyPositionsAsync");
  napi_create_reference(env, a.v[1], 1, &s->pending);
  return undefined(env);
}

// synchronize(h): waits for the substeps and reads issued so far.
napi_value Synchronize(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  const int rc = pbf_synchronize(s->h);
  if (s->pending) {
    napi_delete_reference(env, s->pending);
    s->pending = nullptr;
  }
  return rc ? fail(env, s->h, rc, "synchronize") : undefined(env);
}

// metrics(h) -> {particles, nonfinite, penetrations, errorFlags, maxCompression,
// meanCompression, meanAbsDensityError, maxAbsDensityError, kineticEnergy,
// neighborTotal}.
napi_value Metrics(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Sim* s = sim_arg(env, a.v[0]);
  if (!s) return nullptr;
  pbf_metrics m;
  const int rc = pbf_get_metrics(s->h, &m);
  if (rc) return fail(env, s->h, rc, "metrics");
  napi_value obj;
  napi_create_object(env, &obj);
  set_number(env, obj, "particles", m.particles);
  set_number(env, obj, "nonfinite", m.nonfinite);
  set_number(env, obj, "penetrations", m.penetrations);
  set_number(env, obj, "errorFlags", m.error_flags);
  set_number(env, obj, "maxCompression", m.max_compression);
  set_number(env, obj, "meanCompression", m.mean_compression);
  set_number(env, obj, "meanAbsDensityError", m.mean_abs_density_err);
  set_number(env, obj, "maxAbsDensityError", m.max_abs_density_err);
  set_number(env, obj, "kineticEnergy", m.kinetic_energy);
  set_number(env, obj, "neighborTotal", m.neighbor_total);
  return obj;
}

// ---------------------------------------------------------------- renderer

// rendererCreate(width, height) -> handle: FilteredParticleFluid's depth and
// volume maps (fluid.ts:77-112) without the WebGPU pipelines.
napi_value RendererCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  uint32_t w = 0, h = 0;
  if (!get_u32(env, a.v[0], &w) || !get_u32(env, a.v[1], &h))
    return type_error(env, "rendererCreate(width, height): two whole numbers");
  pbf_renderer* r = nullptr;
  const int rc = pbf_renderer_create(w, h, &r);
  if (rc) return fail(env, nullptr, rc, "rendererCreate");
  Boxed* b = new Boxed{kRenTag, Sim{}, Renderer{r}};
  napi_value ext;
  if (napi_create_external(env, b, finalize_boxed, nullptr, &ext) != napi_ok) {
    pbf_renderer_destroy(r);
    delete b;
    napi_throw_error(env, nullptr, "rendererCreate: napi_create_external failed");
    return nullptr;
  }
  return ext;
}

napi_value RendererDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  pbf_renderer_destroy(r->r);
  r->r = nullptr;
  return undefined(env);
}

// rendererSetConfig(r, {mode, filterSize, particleRadius, opacity, tintColor})
// (fluid.ts:114-133; tintColor as three 0..255 numbers, the GUI's colour).
napi_value RendererSetConfig(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  if (!is_type(env, a.v[1], napi_object)) return type_error(env, "rendererSetConfig(r, options): an object");
  pbf_render_options o;
  o.mode = 0;
  o.filter_size = 32;
  o.particle_radius = 0.02f;
  o.opacity = 0.25f;
  float tint[3] = {6.0f, 105.0f, 217.0f};
  if (!opt_u32(env, a.v[1], "mode", &o.mode) || !opt_u32(env, a.v[1], "filterSize", &o.filter_size) ||
      !opt_number(env, a.v[1], "particleRadius", &o.particle_radius) ||
      !opt_number(env, a.v[1], "opacity", &o.opacity) || !opt_vec3(env, a.v[1], "tintColor", tint))
    return type_error(env, "rendererSetConfig: members must be numbers, tintColor 3 numbers");
  for (int i = 0; i < 3; ++i) o.tint_color[i] = tint[i] / 255.0f;
  const int rc = pbf_renderer_set_config(r->r, &o);
  return rc ? fail(env, nullptr, rc, "rendererSetConfig") : undefined(env);
}

// rendererSetCamera(r, {position[3], view[16], viewInverse[16], projection[16],
// params[4]}): the camera uniform (globalResource.ts:165-181), matrices as
// three.js Matrix4.elements (column-major).
napi_value RendererSetCamera(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  if (!is_type(env, a.v[1], napi_object)) return type_error(env, "rendererSetCamera(r, camera): an object");
  pbf_camera c;
  std::memset(&c, 0, sizeof(c));
  struct Member {
    const char* name;
    float* dst;
    size_t n;
    bool required;
  } members[] = {{"position", c.position, 3, true},
                 {"view", c.view, 16, true},
                 {"viewInverse", c.view_inverse, 16, true},
                 {"projection", c.projection, 16, true},
                 {"params", c.params, 4, false}};
  for (const Member& m : members) {
    napi_value v;
    if (!property(env, a.v[1], m.name, &v)) {
      if (m.required) return type_error(env, (std::string("rendererSetCamera: missing '") + m.name + "'").c_str());
      continue;
    }
    if (!get_floats(env, v, m.dst, m.n))
      return type_error(env, (std::string("rendererSetCamera: '") + m.name + "' has the wrong length").c_str());
  }
  const int rc = pbf_renderer_set_camera(r->r, &c);
  return rc ? fail(env, nullptr, rc, "rendererSetCamera") : undefined(env);
}

// renderSimulation(r, h): ParicleRasterizer + TextureFilter on the
// simulator's position buffer (fluid.ts:150-160).
napi_value RenderSimulation(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  Sim* s = sim_arg(env, a.v[1]);
  if (!s) return nullptr;
  const int rc = pbf_render_simulation(r->r, s->h, nullptr);
  return rc ? fail(env, s->h, rc, "renderSimulation") : undefined(env);
}

uint32_t map_index(napi_env env, napi_value v, bool* ok) {
  uint32_t which = 0;
  *ok = get_u32(env, v, &which) && (which == PBF_RENDER_DEPTH || which == PBF_RENDER_VOLUME);
  return which;
}

// mapSize(r, which) -> [width, height]; which 0 = depth, 1 = volume.
napi_value MapSize(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  bool ok = false;
  const uint32_t which = map_index(env, a.v[1], &ok);
  if (!ok) return type_error(env, "mapSize(r, which): which must be 0 (depth) or 1 (volume)");
  uint32_t w = 0, h = 0;
  const int rc = pbf_renderer_map_size(r->r, which, &w, &h);
  if (rc) return fail(env, nullptr, rc, "mapSize");
  napi_value arr;
  napi_create_array_with_length(env, 2, &arr);
  napi_set_element(env, arr, 0, number(env, w));
  napi_set_element(env, arr, 1, number(env, h));
  return arr;
}

// copyMap(r, which, Float32Array): the depth or volume map, row-major.
napi_value CopyMap(napi_env env, napi_callback_info info) {
  Args a(env, info);
  Renderer* r = renderer_arg(env, a.v[0]);
  if (!r) return nullptr;
  bool ok = false;
  const uint32_t which = map_index(env, a.v[1], &ok);
  if (!ok) return type_error(env, "copyMap(r, which, out): which must be 0 (depth) or 1 (volume)");
  void* p = nullptr;
  size_t len = 0;
  if (!get_typed(env, a.v[2], napi_float32_array, &p, &len)) return type_error(env, "copyMap: out must be a Float32Array");
  const int rc = pbf_renderer_copy_map(r->r, which, static_cast<float*>(p), len * sizeof(float));
  return rc ? fail(env, nullptr, rc, "copyMap") : undefined(env);
}

// ---------------------------------------------------------------- module

napi_value Init(napi_env env, napi_value exports) {
  struct Export {
    const char* name;
    napi_callback fn;
  } table[] = {
      {"create", Create},
      {"destroy", Destroy},
      {"reset", Reset},
      {"setConfig", SetConfig},
      {"getConfig", GetConfig},
      {"voxelizeCube", VoxelizeCube},
      {"voxelizeSphere", VoxelizeSphere},
      {"voxelizeMesh", VoxelizeMesh},
      {"setParticlePosition", SetParticlePosition},
      {"setBoundaryData", SetBoundaryData},
      {"run", Run},
      {"step", Step},
      {"runTimestamp", RunTimestamp},
      {"particleCount", ParticleCount},
      {"setPaused", SetPaused},
      {"isPaused", IsPaused},
      {"copyPositions", CopyPositions},
      {"copyPositionsAsync", CopyPositionsAsync},
      {"synchronize", Synchronize},
      {"metrics", Metrics},
      {"rendererCreate", RendererCreate},
      {"rendererDestroy", RendererDestroy},
      {"rendererSetConfig", RendererSetConfig},
      {"rendererSetCamera", RendererSetCamera},
      {"renderSimulation", RenderSimulation},
      {"mapSize", MapSize},
      {"copyMap", CopyMap},
  };
  for (const Export& e : table) {
    napi_value fn;
    if (napi_create_function(env, e.name, NAPI_AUTO_LENGTH, e.fn, nullptr, &fn) != napi_ok ||
        napi_set_named_property(env, exports, e.name, fn) != napi_ok) {
      napi_throw_error(env, nullptr, "pbf_gb300 addon: could not register its exports");
      return nullptr;
    }
  }
  napi_set_named_property(env, exports, "abiVersion", number(env, pbf_abi_version()));
  return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
