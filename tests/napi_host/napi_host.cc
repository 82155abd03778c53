// napi_host.cc - a stand-in for Node that loads the pbf_gb300 addon
// (webgpu-fluid-simulation_gb300/napi/pbf_addon.cc) with dlopen, registers
// it through napi_register_module_v1 and calls its exports the way pbf.ts
// does.  It implements the Node-API subset of node_api.h over a small value
// model (numbers, strings, objects, arrays, typed arrays, functions,
// externals, references, a pending exception) and a collector that runs an
// External's finaliser once nothing references it.
//
//   napi_host ADDON.so cpu   argument checks and error paths that need no GPU
//   napi_host ADDON.so gpu   the Cube Drop flow, mesh seeding and the renderer
//                            through the addon, checked against the C ABI
//
// Prints one line and exits 0 when every check holds.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "node_api.h"
#include "pbf_gb300.h"

// ---------------------------------------------------------------- value model

struct napi_value__ {
  napi_valuetype type = napi_undefined;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::map<std::string, napi_value> props;
  bool is_array = false;
  std::vector<napi_value> elems;
  bool is_typed = false;
  napi_typedarray_type ta = napi_float32_array;
  std::vector<double> store;  // typed-array bytes (8-byte aligned)
  size_t length = 0;
  napi_callback cb = nullptr;
  void* cb_data = nullptr;
  void* ext = nullptr;
  napi_finalize fin = nullptr;
  void* hint = nullptr;
  uint32_t refs = 0;
  bool finalized = false;
};

struct napi_ref__ {
  napi_value v;
  uint32_t count;
};

struct napi_env__ {
  std::vector<std::unique_ptr<napi_value__>> heap;
  std::vector<std::unique_ptr<napi_ref__>> refs;
  napi_value exception = nullptr;
  napi_value undef = nullptr;
  napi_value null = nullptr;
  napi_value t = nullptr;
  napi_value f = nullptr;
  int finalized = 0;
};

struct napi_callback_info__ {
  size_t argc;
  napi_value* argv;
  void* data;
};

static napi_value alloc(napi_env env, napi_valuetype t) {
  env->heap.emplace_back(new napi_value__());
  napi_value v = env->heap.back().get();
  v->type = t;
  return v;
}

static size_t elem_size(napi_typedarray_type t) {
  switch (t) {
    case napi_int8_array:
    case napi_uint8_array:
    case napi_uint8_clamped_array: return 1;
    case napi_int16_array:
    case napi_uint16_array: return 2;
    case napi_int32_array:
    case napi_uint32_array:
    case napi_float32_array: return 4;
    default: return 8;
  }
}

static napi_value typed(napi_env env, napi_typedarray_type t, size_t n) {
  napi_value v = alloc(env, napi_object);
  v->is_typed = true;
  v->ta = t;
  v->length = n;
  v->store.assign((n * elem_size(t) + 7) / 8 + 1, 0.0);
  return v;
}

template <class T>
static T* data_of(napi_value v) {
  return reinterpret_cast<T*>(v->store.data());
}

extern "C" {

napi_status napi_get_undefined(napi_env env, napi_value* r) {
  *r = env->undef;
  return napi_ok;
}
napi_status napi_get_boolean(napi_env env, bool value, napi_value* r) {
  *r = value ? env->t : env->f;
  return napi_ok;
}
napi_status napi_create_double(napi_env env, double value, napi_value* r) {
  *r = alloc(env, napi_number);
  (*r)->num = value;
  return napi_ok;
}
napi_status napi_create_object(napi_env env, napi_value* r) {
  *r = alloc(env, napi_object);
  return napi_ok;
}
napi_status napi_create_array_with_length(napi_env env, size_t length, napi_value* r) {
  *r = alloc(env, napi_object);
  (*r)->is_array = true;
  (*r)->elems.assign(length, env->undef);
  return napi_ok;
}
napi_status napi_create_function(napi_env env, const char* name, size_t, napi_callback cb, void* data, napi_value* r) {
  if (!cb || !r) return napi_invalid_arg;
  *r = alloc(env, napi_function);
  (*r)->cb = cb;
  (*r)->cb_data = data;
  (*r)->str = name ? name : "";
  return napi_ok;
}
napi_status napi_create_external(napi_env env, void* data, napi_finalize fin, void* hint, napi_value* r) {
  *r = alloc(env, napi_external);
  (*r)->ext = data;
  (*r)->fin = fin;
  (*r)->hint = hint;
  return napi_ok;
}
napi_status napi_typeof(napi_env, napi_value v, napi_valuetype* r) {
  if (!v) return napi_invalid_arg;
  *r = v->type;
  return napi_ok;
}
napi_status napi_get_value_double(napi_env, napi_value v, double* r) {
  if (!v || v->type != napi_number) return napi_number_expected;
  *r = v->num;
  return napi_ok;
}
napi_status napi_get_value_bool(napi_env, napi_value v, bool* r) {
  if (!v || v->type != napi_boolean) return napi_boolean_expected;
  *r = v->b;
  return napi_ok;
}
napi_status napi_get_value_external(napi_env, napi_value v, void** r) {
  if (!v || v->type != napi_external) return napi_invalid_arg;
  *r = v->ext;
  return napi_ok;
}
napi_status napi_get_value_string_utf8(napi_env, napi_value v, char* buf, size_t bufsize, size_t* r) {
  if (!v || v->type != napi_string) return napi_string_expected;
  if (!buf) {
    if (r) *r = v->str.size();
    return napi_ok;
  }
  if (bufsize == 0) return napi_invalid_arg;
  const size_t n = std::min(bufsize - 1, v->str.size());
  std::memcpy(buf, v->str.data(), n);
  buf[n] = '\0';
  if (r) *r = n;
  return napi_ok;
}
napi_status napi_is_array(napi_env, napi_value v, bool* r) {
  *r = v && v->is_array;
  return napi_ok;
}
napi_status napi_get_array_length(napi_env, napi_value v, uint32_t* r) {
  if (!v || !v->is_array) return napi_array_expected;
  *r = static_cast<uint32_t>(v->elems.size());
  return napi_ok;
}
napi_status napi_get_element(napi_env env, napi_value v, uint32_t i, napi_value* r) {
  if (!v || v->type != napi_object) return napi_object_expected;
  *r = (v->is_array && i < v->elems.size()) ? v->elems[i] : env->undef;
  return napi_ok;
}
napi_status napi_set_element(napi_env, napi_value v, uint32_t i, napi_value e) {
  if (!v || !v->is_array) return napi_object_expected;
  if (i >= v->elems.size()) v->elems.resize(i + 1, nullptr);
  v->elems[i] = e;
  return napi_ok;
}
napi_status napi_is_typedarray(napi_env, napi_value v, bool* r) {
  *r = v && v->is_typed;
  return napi_ok;
}
napi_status napi_get_typedarray_info(napi_env env, napi_value v, napi_typedarray_type* type, size_t* length,
                                     void** data, napi_value* ab, size_t* off) {
  if (!v || !v->is_typed) return napi_invalid_arg;
  if (type) *type = v->ta;
  if (length) *length = v->length;
  if (data) *data = v->store.data();
  if (ab) *ab = env->undef;
  if (off) *off = 0;
  return napi_ok;
}
napi_status napi_has_named_property(napi_env, napi_value v, const char* name, bool* r) {
  if (!v || (v->type != napi_object && v->type != napi_function)) return napi_object_expected;
  *r = v->props.count(name) != 0;
  return napi_ok;
}
napi_status napi_get_named_property(napi_env env, napi_value v, const char* name, napi_value* r) {
  if (!v || (v->type != napi_object && v->type != napi_function)) return napi_object_expected;
  auto it = v->props.find(name);
  *r = it == v->props.end() ? env->undef : it->second;
  return napi_ok;
}
napi_status napi_set_named_property(napi_env, napi_value v, const char* name, napi_value e) {
  if (!v || (v->type != napi_object && v->type != napi_function)) return napi_object_expected;
  v->props[name] = e;
  return napi_ok;
}
napi_status napi_get_cb_info(napi_env env, napi_callback_info info, size_t* argc, napi_value* argv, napi_value* self,
                             void** data) {
  if (argc) {
    for (size_t i = 0; i < *argc; ++i) argv[i] = i < info->argc ? info->argv[i] : env->undef;
    *argc = info->argc;
  }
  if (self) *self = env->undef;
  if (data) *data = info->data;
  return napi_ok;
}
static napi_status throw_with(napi_env env, const char* kind, const char* code, const char* msg) {
  if (env->exception) return napi_pending_exception;
  napi_value e = alloc(env, napi_object);
  napi_value s = alloc(env, napi_string);
  s->str = msg ? msg : "";
  e->props["message"] = s;
  napi_value k = alloc(env, napi_string);
  k->str = kind;
  e->props["name"] = k;
  if (code) {
    napi_value c = alloc(env, napi_string);
    c->str = code;
    e->props["code"] = c;
  }
  env->exception = e;
  return napi_ok;
}
napi_status napi_throw_error(napi_env env, const char* code, const char* msg) {
  return throw_with(env, "Error", code, msg);
}
napi_status napi_throw_type_error(napi_env env, const char* code, const char* msg) {
  return throw_with(env, "TypeError", code, msg);
}
napi_status napi_create_reference(napi_env env, napi_value v, uint32_t count, napi_ref* r) {
  if (!v) return napi_invalid_arg;
  env->refs.emplace_back(new napi_ref__{v, count});
  v->refs += count;
  *r = env->refs.back().get();
  return napi_ok;
}
napi_status napi_delete_reference(napi_env env, napi_ref ref) {
  for (auto& p : env->refs)
    if (p.get() == ref) {
      ref->v->refs -= ref->count;
      p.reset();
      return napi_ok;
    }
  return napi_invalid_arg;
}

}  // extern "C"

// ---------------------------------------------------------------- host helpers

static int g_failures = 0;
#define CHECK(cond, ...)                                   \
  do {                                                     \
    if (!(cond)) {                                         \
      ++g_failures;                                        \
      std::fprintf(stderr, "check failed (line %d): ", __LINE__); \
      std::fprintf(stderr, __VA_ARGS__);                   \
      std::fprintf(stderr, "\n");                          \
    }                                                      \
  } while (0)

struct Host {
  napi_env__ env_;
  napi_env env = &env_;
  napi_value exports = nullptr;

  Host() {
    env->undef = alloc(env, napi_undefined);
    env->null = alloc(env, napi_null);
    env->t = alloc(env, napi_boolean);
    env->t->b = true;
    env->f = alloc(env, napi_boolean);
  }
  // What Node does with live Externals when the environment goes away.
  ~Host() {
    for (auto& v : env->heap) collect(v.get(), true);
  }

  napi_value num(double x) {
    napi_value v;
    napi_create_double(env, x, &v);
    return v;
  }
  napi_value str(const std::string& s) {
    napi_value v = alloc(env, napi_string);
    v->str = s;
    return v;
  }
  napi_value arr(std::initializer_list<double> xs) {
    napi_value v;
    napi_create_array_with_length(env, 0, &v);
    for (double x : xs) v->elems.push_back(num(x));
    return v;
  }
  napi_value arr16(const double* m) {
    napi_value v;
    napi_create_array_with_length(env, 0, &v);
    for (int i = 0; i < 16; ++i) v->elems.push_back(num(m[i]));
    return v;
  }
  napi_value f32(size_t n, const float* src = nullptr) {
    napi_value v = typed(env, napi_float32_array, n);
    if (src) std::memcpy(data_of<float>(v), src, n * sizeof(float));
    return v;
  }
  napi_value obj(std::initializer_list<std::pair<const char*, napi_value>> kv) {
    napi_value v = alloc(env, napi_object);
    for (auto& p : kv) v->props[p.first] = p.second;
    return v;
  }

  // Calls exports[name](args...); returns the result, or nullptr with the
  // thrown Error's name, code and message in err_*.
  std::string err_name, err_code, err_msg;
  napi_value call(const char* name, std::vector<napi_value> args) {
    err_name.clear();
    err_code.clear();
    err_msg.clear();
    auto it = exports->props.find(name);
    if (it == exports->props.end() || it->second->type != napi_function) {
      err_name = "ReferenceError";
      err_msg = std::string("no export ") + name;
      return nullptr;
    }
    napi_callback_info__ info{args.size(), args.data(), it->second->cb_data};
    napi_value r = it->second->cb(env, &info);
    if (env->exception) {
      napi_value e = env->exception;
      env->exception = nullptr;
      err_name = e->props["name"]->str;
      if (e->props.count("code")) err_code = e->props["code"]->str;
      err_msg = e->props["message"]->str;
      return nullptr;
    }
    return r ? r : env->undef;
  }
  bool threw(const char* name, const char* code = nullptr) const {
    return err_name == name && (!code || err_code == code);
  }

  // The collector: finalises an External that nothing references.
  bool collect(napi_value v, bool teardown = false) {
    if (v->type != napi_external || v->finalized) return false;
    if (v->refs && !teardown) return false;
    v->finalized = true;
    if (v->fin) v->fin(env, v->ext, v->hint);
    ++env->finalized;
    return true;
  }
};

static double get_num(napi_value v) { return v && v->type == napi_number ? v->num : std::nan(""); }
static double prop_num(napi_value o, const char* k) {
  return o && o->props.count(k) ? get_num(o->props[k]) : std::nan("");
}

// ---------------------------------------------------------------- camera

// three.js PerspectiveCamera with the reverse-Z projection of
// src/controller.ts:15-35 (fov 50, near 0.1, far 30) at `eye` looking at
// the origin; column-major doubles (Matrix4.elements).
struct Cam {
  double view[16], world[16], proj[16], pos[3], params[4];
};
static Cam reference_camera(double w, double h, double ex, double ey, double ez) {
  Cam c{};
  const double fov = 50.0, nearp = 0.1, farp = 30.0, aspect = w / h;
  double z[3] = {ex, ey, ez};
  double zl = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
  for (double& a : z) a /= zl;
  double x[3] = {1.0 * z[2] - 0.0 * z[1], 0.0 * z[0] - 0.0 * z[2], 0.0 * z[1] - 1.0 * z[0]};  // up x z, up = +y
  double xl = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  for (double& a : x) a /= xl;
  double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  const double e[3] = {ex, ey, ez};
  for (int r = 0; r < 3; ++r) {
    c.world[0 * 4 + r] = x[r];
    c.world[1 * 4 + r] = y[r];
    c.world[2 * 4 + r] = z[r];
    c.world[3 * 4 + r] = e[r];
  }
  c.world[15] = 1.0;
  // inverse of a rigid transform: R^T, -R^T e
  for (int r = 0; r < 3; ++r) {
    const double* axis = r == 0 ? x : (r == 1 ? y : z);
    for (int k = 0; k < 3; ++k) c.view[k * 4 + r] = axis[k];
    c.view[12 + r] = -(axis[0] * e[0] + axis[1] * e[1] + axis[2] * e[2]);
  }
  c.view[15] = 1.0;
  const double top = nearp * std::tan(M_PI / 180.0 * 0.5 * fov), height = 2.0 * top, width = aspect * height;
  c.proj[0] = 2.0 * nearp / width;
  c.proj[5] = 2.0 * nearp / height;
  c.proj[10] = nearp / (farp - nearp);
  c.proj[11] = -1.0;
  c.proj[14] = farp * nearp / (farp - nearp);
  for (int i = 0; i < 3; ++i) c.pos[i] = e[i];
  c.params[0] = aspect * height / nearp;
  c.params[1] = -height / nearp;
  c.params[2] = (farp - nearp) / (nearp * farp);
  c.params[3] = 1.0 / farp;
  return c;
}

// ---------------------------------------------------------------- checks

static const char* kExports[] = {"create", "destroy", "reset", "setConfig", "getConfig", "voxelizeCube",
                                 "voxelizeSphere", "voxelizeMesh", "setParticlePosition", "setBoundaryData", "run",
                                 "step", "runTimestamp", "particleCount", "setPaused", "isPaused", "copyPositions",
                                 "copyPositionsAsync", "synchronize", "metrics", "rendererCreate",
                                 "rendererDestroy", "rendererSetConfig", "rendererSetCamera", "renderSimulation",
                                 "mapSize", "copyMap"};

static void cpu_checks(Host& H) {
  for (const char* n : kExports)
    CHECK(H.exports->props.count(n) && H.exports->props[n]->type == napi_function, "export %s missing", n);
  CHECK(get_num(H.exports->props["abiVersion"]) == PBF_ABI_VERSION, "abiVersion");

  // wrong argument types throw TypeError before the library is called
  H.call("create", {H.num(5)});
  CHECK(H.threw("TypeError", "ERR_INVALID_ARG_TYPE"), "create(5): %s %s", H.err_name.c_str(), H.err_msg.c_str());
  H.call("create", {H.obj({{"particleRadius", H.str("big")}})});
  CHECK(H.threw("TypeError"), "create({particleRadius: 'big'})");
  H.call("create", {H.obj({{"domainMax", H.arr({1.0, 2.0})}})});
  CHECK(H.threw("TypeError"), "create({domainMax: [1, 2]})");
  H.call("voxelizeCube", {H.env->undef, H.arr({0, 0, 0}), H.arr({1, 1, 1})});
  CHECK(H.threw("TypeError") && H.err_msg.find("simulator handle") != std::string::npos, "voxelizeCube(undefined)");
  H.call("step", {H.obj({})});
  CHECK(H.threw("TypeError"), "step({})");
  H.call("rendererCreate", {H.str("a"), H.num(2)});
  CHECK(H.threw("TypeError"), "rendererCreate('a', 2)");
  H.call("copyMap", {H.num(1), H.num(0), H.f32(4)});
  CHECK(H.threw("TypeError"), "copyMap(1, ...)");

  // an invalid configuration is refused by pbf_create before any device call
  H.call("create", {H.obj({{"kernelRadius", H.num(-1.0)}})});
  CHECK(H.threw("Error", "PBF_EINVAL") && H.err_msg.find("create failed") == 0, "create({kernelRadius: -1}): %s %s",
        H.err_code.c_str(), H.err_msg.c_str());
  H.call("create", {H.obj({{"domainMin", H.arr({0, 0, 0})}, {"domainMax", H.arr({1, 0, 1})}})});
  CHECK(H.threw("Error", "PBF_EINVAL"), "create with an empty domain");

  // with or without a device, create() either gives a handle or throws PBF_ECUDA
  napi_value h = H.call("create", {});
  if (h) {
    CHECK(h->type == napi_external, "create() result");
    H.call("destroy", {h});
  } else {
    CHECK(H.threw("Error", "PBF_ECUDA"), "create() without a device: %s %s", H.err_code.c_str(), H.err_msg.c_str());
  }
}

static void gpu_checks(Host& H) {
  // ---- Cube Drop (src/controller.ts:202-208, 343-347, 375-376)
  napi_value h = H.call("create", {});
  CHECK(h && h->type == napi_external, "create(): %s", H.err_msg.c_str());
  if (!h) return;
  CHECK(get_num(H.call("particleCount", {h})) == 0.0, "particleCount before seeding");
  napi_value mx = H.f32(3);
  data_of<float>(mx)[0] = 0.65f, data_of<float>(mx)[1] = 0.85f, data_of<float>(mx)[2] = 0.65f;
  napi_value added = H.call("voxelizeCube", {h, H.arr({0.15, 0.35, 0.15}), mx});
  CHECK(get_num(added) == 41.0 * 41.0 * 41.0, "voxelizeCube added %g", get_num(added));
  H.call("setParticlePosition", {h});
  CHECK(H.err_name.empty(), "setParticlePosition: %s", H.err_msg.c_str());
  napi_value conf = H.obj({{"iteration", H.num(5)}, {"XSPH", H.num(0.01)}, {"vorticity", H.num(0.1)},
                           {"surfaceTension", H.num(0.5)}, {"gravity", H.num(9.8)}});
  H.call("setConfig", {h, conf});
  CHECK(H.err_name.empty(), "setConfig: %s", H.err_msg.c_str());
  napi_value back = H.call("getConfig", {h});
  CHECK(prop_num(back, "iteration") == 5.0 && prop_num(back, "XSPH") == (double)0.01f &&
            prop_num(back, "gravity") == (double)9.8f,
        "getConfig round trip");
  H.call("setConfig", {h, H.obj({{"iteration", H.num(5)}})});
  CHECK(H.threw("TypeError") && H.err_msg.find("XSPH") != std::string::npos, "setConfig without XSPH");
  H.call("setConfig", {h, H.obj({{"iteration", H.num(2.5)}, {"XSPH", H.num(0)}, {"vorticity", H.num(0)},
                                 {"surfaceTension", H.num(0)}, {"gravity", H.num(0)}})});
  CHECK(H.threw("TypeError"), "setConfig with 2.5 iterations");

  const uint32_t n = 41u * 41u * 41u;
  napi_value async_out = H.f32(4 * (size_t)n);
  for (int f = 0; f < 20; ++f) {
    H.call("step", {h, H.num(1)});
    CHECK(H.err_name.empty(), "step: %s", H.err_msg.c_str());
  }
  H.call("copyPositionsAsync", {h, async_out});
  CHECK(H.err_name.empty(), "copyPositionsAsync: %s", H.err_msg.c_str());
  CHECK(async_out->refs == 1, "the addon pins the array of an asynchronous read");
  H.call("synchronize", {h});
  CHECK(H.err_name.empty() && async_out->refs == 0, "synchronize releases the array");
  napi_value sync_out = H.f32(4 * (size_t)n);
  H.call("copyPositions", {h, sync_out});
  CHECK(H.err_name.empty(), "copyPositions: %s", H.err_msg.c_str());
  CHECK(std::memcmp(data_of<float>(async_out), data_of<float>(sync_out), 16 * (size_t)n) == 0,
        "asynchronous and synchronous reads differ");
  H.call("copyPositions", {h, H.f32(8)});
  CHECK(H.threw("TypeError"), "copyPositions into a short array");
  unsigned bad = 0;
  float ymin = 1e30f;
  for (uint32_t i = 0; i < n; ++i) {
    const float* q = data_of<float>(sync_out) + 4 * (size_t)i;
    if (!std::isfinite(q[0]) || !std::isfinite(q[1]) || !std::isfinite(q[2])) ++bad;
    ymin = std::min(ymin, q[1]);
  }
  CHECK(bad == 0 && ymin < 0.35f, "positions: %u non-finite, lowest y %g", bad, ymin);
  napi_value m = H.call("metrics", {h});
  CHECK(prop_num(m, "particles") == n && prop_num(m, "nonfinite") == 0 && prop_num(m, "errorFlags") == 0,
        "metrics");
  napi_value ts = H.call("runTimestamp", {h});
  CHECK(ts && ts->is_array && ts->elems.size() == 4 && get_num(ts->elems[2]) > 0.0, "runTimestamp");

  // pause (SPH.ts:82-84): a paused simulator does not move
  H.call("setPaused", {h, H.env->t});
  CHECK(H.call("isPaused", {h}) == H.env->t, "isPaused");
  H.call("step", {h, H.num(3)});
  napi_value paused_out = H.f32(4 * (size_t)n);
  H.call("copyPositions", {h, paused_out});
  H.call("copyPositions", {h, sync_out});
  CHECK(std::memcmp(data_of<float>(paused_out), data_of<float>(sync_out), 16 * (size_t)n) == 0, "paused step moved");
  H.call("setPaused", {h, H.num(0)});
  CHECK(H.threw("TypeError"), "setPaused(h, 0)");
  H.call("setPaused", {h, H.env->f});

  // errors the reference throws: malformed boundary text, too many particles
  H.call("setBoundaryData", {h, H.str("1 2 3\nnot a volume map")});
  CHECK(H.threw("Error", "PBF_EFORMAT") && H.err_msg.find("Boundary") != std::string::npos,
        "setBoundaryData: %s %s", H.err_code.c_str(), H.err_msg.c_str());
  napi_value small = H.call("create", {H.obj({{"maxParticles", H.num(1000)}})});
  CHECK(small != nullptr, "create({maxParticles: 1000})");
  if (small) {
    H.call("voxelizeCube", {small, H.arr({0.1, 0.1, 0.1}), H.arr({0.5, 0.5, 0.5})});
    H.call("setParticlePosition", {small});
    CHECK(H.threw("Error", "PBF_ECAPACITY") && H.err_msg.find("To Many Particles") != std::string::npos,
          "setParticlePosition over capacity: %s", H.err_msg.c_str());
    // dropped without destroy: the collector's finaliser frees it
    const int before = H.env->finalized;
    CHECK(H.collect(small) && H.env->finalized == before + 1, "finaliser of a dropped handle");
  }

  // ---- voxelizeMesh: indexed and non-indexed geometry give the C ABI's points
  {
    const float cube[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    const uint32_t tri[12][3] = {{0, 2, 1}, {0, 3, 2}, {4, 5, 6}, {4, 6, 7}, {0, 1, 5}, {0, 5, 4},
                                 {2, 3, 7}, {2, 7, 6}, {1, 2, 6}, {1, 6, 5}, {0, 4, 7}, {0, 7, 3}};
    const double world[16] = {0.1, 0, 0, 0, 0, 0.08, 0, 0, 0, 0, 0.125, 0, 0.5, 0.3, 0.5, 1};
    napi_value pos = H.f32(24, &cube[0][0]);
    napi_value idx = typed(H.env, napi_uint32_array, 36);
    std::memcpy(data_of<uint32_t>(idx), &tri[0][0], sizeof(tri));
    std::vector<float> flat(108);
    for (int t = 0; t < 12; ++t)
      for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) flat[9 * t + 3 * k + a] = cube[tri[t][k]][a];
    // the handle's lattice spacing is 2 r with r the float 0.006f
    uint32_t want = 0, got = 0;
    int rc = pbf_voxelize_mesh_points(&cube[0][0], 8, &tri[0][0], 12, world, (double)0.006f, nullptr, 0, &want);
    CHECK(rc == PBF_ECAPACITY && want > 1000, "pbf_voxelize_mesh_points (count): rc %d, %u points", rc, want);
    std::vector<float> pts(4 * (size_t)want);
    rc = pbf_voxelize_mesh_points(&cube[0][0], 8, &tri[0][0], 12, world, (double)0.006f, pts.data(), want, &got);
    CHECK(rc == PBF_OK && got == want, "pbf_voxelize_mesh_points: rc %d, %u points", rc, got);
    napi_value hm = H.call("create", {});
    napi_value a1 = H.call("voxelizeMesh", {hm, pos, idx, H.arr16(world)});
    napi_value a2 = H.call("voxelizeMesh", {hm, H.f32(108, flat.data()), H.env->null, H.arr16(world)});
    CHECK(get_num(a1) == want && get_num(a2) == want, "voxelizeMesh added %g / %g, C ABI %u", get_num(a1),
          get_num(a2), want);
    H.call("voxelizeMesh", {hm, pos, idx, H.arr({1, 0, 0})});
    CHECK(H.threw("TypeError"), "voxelizeMesh with a 3-element matrix");
    napi_value sphere = H.call("voxelizeSphere", {hm, H.arr({0.5, 0.5, 0.5}), H.num(0.05)});
    CHECK(get_num(sphere) > 100, "voxelizeSphere added %g", get_num(sphere));
    H.call("setParticlePosition", {hm});
    CHECK(get_num(H.call("particleCount", {hm})) == 2.0 * want + get_num(sphere), "mesh handle count");
    H.call("destroy", {hm});
    H.call("run", {hm});
    CHECK(H.threw("Error", "PBF_ESTATE"), "run after destroy");
  }

  // ---- renderer: the addon's maps equal the C ABI's for the same camera
  {
    const uint32_t W = 320, Ht = 180;
    const Cam c = reference_camera(W, Ht, 1.6, 1.4, 1.2);
    napi_value r = H.call("rendererCreate", {H.num(W), H.num(Ht)});
    CHECK(r != nullptr, "rendererCreate: %s", H.err_msg.c_str());
    H.call("rendererSetConfig", {r, H.obj({{"filterSize", H.num(16)}, {"particleRadius", H.num(0.02)},
                                           {"tintColor", H.arr({6, 105, 217})}})});
    CHECK(H.err_name.empty(), "rendererSetConfig: %s", H.err_msg.c_str());
    float viewf[16];
    for (int i = 0; i < 16; ++i) viewf[i] = (float)c.view[i];
    napi_value camobj = H.obj({{"position", H.arr({c.pos[0], c.pos[1], c.pos[2]})},
                               {"view", H.f32(16, viewf)},
                               {"viewInverse", H.arr16(c.world)},
                               {"projection", H.arr16(c.proj)},
                               {"params", H.arr({c.params[0], c.params[1], c.params[2], c.params[3]})}});
    H.call("renderSimulation", {r, h});
    CHECK(H.threw("Error"), "renderSimulation before a camera");
    H.call("rendererSetCamera", {r, H.obj({{"position", H.arr({0, 0, 0})}})});
    CHECK(H.threw("TypeError") && H.err_msg.find("view") != std::string::npos, "camera without view");
    H.call("rendererSetCamera", {r, camobj});
    CHECK(H.err_name.empty(), "rendererSetCamera: %s", H.err_msg.c_str());
    H.call("renderSimulation", {r, h});
    CHECK(H.err_name.empty(), "renderSimulation: %s", H.err_msg.c_str());
    napi_value size = H.call("mapSize", {r, H.num(PBF_RENDER_VOLUME)});
    CHECK(size && size->elems.size() == 2 && get_num(size->elems[0]) == W / 2 && get_num(size->elems[1]) == Ht / 2,
          "mapSize(volume)");
    napi_value depth = H.f32((size_t)W * Ht), volume = H.f32((size_t)W * Ht / 4);
    H.call("copyMap", {r, H.num(PBF_RENDER_DEPTH), depth});
    H.call("copyMap", {r, H.num(PBF_RENDER_VOLUME), volume});
    CHECK(H.err_name.empty(), "copyMap: %s", H.err_msg.c_str());

    // the same frame through the C ABI directly
    pbf_renderer* pr = nullptr;
    pbf_render_options o{};
    o.filter_size = 16;
    o.particle_radius = 0.02f;
    o.opacity = 0.25f;
    pbf_camera pc{};
    for (int i = 0; i < 3; ++i) pc.position[i] = (float)c.pos[i];
    for (int i = 0; i < 16; ++i) {
      pc.view[i] = (float)c.view[i];
      pc.view_inverse[i] = (float)c.world[i];
      pc.projection[i] = (float)c.proj[i];
    }
    for (int i = 0; i < 4; ++i) pc.params[i] = (float)c.params[i];
    std::vector<float> d2((size_t)W * Ht), v2((size_t)W * Ht / 4);
    {
      // the addon's particle positions, uploaded into a handle of the host's
      // own and rendered by the C ABI renderer
      napi_value host_pos = H.f32(4 * (size_t)n);
      H.call("copyPositions", {h, host_pos});
      pbf_handle* tmp = nullptr;
      pbf_config cfg;
      pbf_config_default(&cfg);
      CHECK(pbf_create(&cfg, &tmp) == PBF_OK, "pbf_create");
      CHECK(pbf_set_particles(tmp, data_of<float>(host_pos), n) == PBF_OK, "pbf_set_particles");
      const float* dpos = pbf_position_device(tmp);
      CHECK(pbf_renderer_create(W, Ht, &pr) == PBF_OK && pbf_renderer_set_config(pr, &o) == PBF_OK &&
                pbf_renderer_set_camera(pr, &pc) == PBF_OK,
            "C ABI renderer");
      CHECK(pbf_render(pr, dpos, n, nullptr, pbf_stream(tmp)) == PBF_OK, "pbf_render");
      CHECK(pbf_renderer_copy_map(pr, PBF_RENDER_DEPTH, d2.data(), d2.size() * 4) == PBF_OK &&
                pbf_renderer_copy_map(pr, PBF_RENDER_VOLUME, v2.data(), v2.size() * 4) == PBF_OK,
            "pbf_renderer_copy_map");
      pbf_renderer_destroy(pr);
      pbf_destroy(tmp);
    }
    size_t covered = 0;
    for (size_t i = 0; i < d2.size(); ++i) covered += d2[i] > 0.0f;
    CHECK(covered > 1000, "covered pixels %zu", covered);
    CHECK(std::memcmp(data_of<float>(depth), d2.data(), d2.size() * 4) == 0, "depth map differs from the C ABI's");
    CHECK(std::memcmp(data_of<float>(volume), v2.data(), v2.size() * 4) == 0, "volume map differs from the C ABI's");
    H.call("rendererDestroy", {r});
    H.call("copyMap", {r, H.num(0), depth});
    CHECK(H.threw("Error", "PBF_ESTATE"), "copyMap after rendererDestroy");
  }
  H.call("destroy", {h});
  H.call("destroy", {h});
  CHECK(H.threw("Error", "PBF_ESTATE"), "second destroy");
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: napi_host ADDON.so cpu|gpu\n");
    return 2;
  }
  void* lib = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);
  if (!lib) {
    std::fprintf(stderr, "dlopen: %s\n", dlerror());
    return 2;
  }
  using Reg = napi_value (*)(napi_env, napi_value);
  Reg reg = reinterpret_cast<Reg>(dlsym(lib, "napi_register_module_v1"));
  if (!reg) {
    std::fprintf(stderr, "no napi_register_module_v1 in %s\n", argv[1]);
    return 2;
  }
  int finalized = 0;
  {
    Host H;
    napi_value exports;
    napi_create_object(H.env, &exports);
    H.exports = reg(H.env, exports);
    CHECK(H.exports == exports && !H.env->exception, "module registration");
    if (std::strcmp(argv[2], "gpu") == 0)
      gpu_checks(H);
    else
      cpu_checks(H);
    finalized = H.env->finalized;
  }
  std::printf("napi_host %s: %d failed checks, %d externals finalised before teardown\n", argv[2], g_failures,
              finalized);
  return g_failures == 0 ? 0 : 1;
}
