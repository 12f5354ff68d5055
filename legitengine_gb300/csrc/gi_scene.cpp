// gi_scene.cpp -- scene files of the reference (bin/data/Scenes/*.json) as
// world-space triangle meshes for gi_gbuffer_mesh / gi_shadow_map_mesh.
//
// The reference loads a scene in Scene.h:55-117: every entry of "meshes" is an
// OBJ file read by tinyobjloader 1.4 with triangulation (Mesh.h:14-57: positions
// times the entry's "scale", the corner's normal or (1, 0, 0) without one);
// every entry of "objects" places a mesh by translate(pos) * rotate(|angle|,
// angle / |angle|) (the rotation only for |angle| > 1e-3) with "albedoColor" and
// "emissiveColor", which the G-buffer pass extends with alpha 1
// (SSVGIRenderer.h:142-143).  Vectors read as ReadJsonVec3f does
// (main.cpp:24-27): a missing member or component is 0.  The file may hold C and
// C++ comments, as jsoncpp accepts.  An object whose mesh is not declared is
// skipped (Scene.h:95-99).
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <locale>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "gi_internal.h"

namespace gi {
namespace {

// ---- JSON ------------------------------------------------------------------
struct JVal {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;

  const JVal* get(const char* key) const {
    if (kind != Obj) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
  std::string get_string(const char* key, const char* fallback) const {
    const JVal* v = get(key);
    return (v && v->kind == Str) ? v->str : std::string(fallback);
  }
};

// Recursive-descent parser for the JSON the scene files use, skipping // and
// /* */ comments between tokens.
class JsonParser {
 public:
  explicit JsonParser(const std::string& text) : s_(text) {}

  JVal Parse() {
    JVal v = Value(0);
    Space();
    if (i_ != s_.size()) Fail("unexpected text after the document");
    return v;
  }

 private:
  [[noreturn]] void Fail(const char* what) const {
    throw std::runtime_error(std::string("scene file: ") + what + " at offset " + std::to_string(i_));
  }

  void Space() {
    for (;;) {
      while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) i_++;
      if (s_.compare(i_, 2, "//") == 0) {
        while (i_ < s_.size() && s_[i_] != '\n') i_++;
      } else if (s_.compare(i_, 2, "/*") == 0) {
        const size_t e = s_.find("*/", i_ + 2);
        if (e == std::string::npos) Fail("unterminated comment");
        i_ = e + 2;
      } else {
        return;
      }
    }
  }

  JVal Value(int depth) {
    if (depth > 64) Fail("nesting too deep");
    Space();
    if (i_ >= s_.size()) Fail("unexpected end");
    const char c = s_[i_];
    JVal v;
    if (c == '{') {
      v.kind = JVal::Obj;
      i_++;
      Space();
      if (i_ < s_.size() && s_[i_] == '}') {
        i_++;
        return v;
      }
      for (;;) {
        Space();
        if (i_ >= s_.size() || s_[i_] != '"') Fail("expected a member name");
        std::string key = String();
        Space();
        if (i_ >= s_.size() || s_[i_] != ':') Fail("expected ':'");
        i_++;
        v.obj.emplace_back(std::move(key), Value(depth + 1));
        Space();
        if (i_ < s_.size() && s_[i_] == ',') {
          i_++;
          continue;
        }
        if (i_ < s_.size() && s_[i_] == '}') {
          i_++;
          return v;
        }
        Fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      v.kind = JVal::Arr;
      i_++;
      Space();
      if (i_ < s_.size() && s_[i_] == ']') {
        i_++;
        return v;
      }
      for (;;) {
        v.arr.push_back(Value(depth + 1));
        Space();
        if (i_ < s_.size() && s_[i_] == ',') {
          i_++;
          continue;
        }
        if (i_ < s_.size() && s_[i_] == ']') {
          i_++;
          return v;
        }
        Fail("expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.kind = JVal::Str;
      v.str = String();
      return v;
    }
    if (s_.compare(i_, 4, "true") == 0) {
      i_ += 4;
      v.kind = JVal::Bool;
      v.b = true;
      return v;
    }
    if (s_.compare(i_, 5, "false") == 0) {
      i_ += 5;
      v.kind = JVal::Bool;
      return v;
    }
    if (s_.compare(i_, 4, "null") == 0) {
      i_ += 4;
      return v;
    }
    // Numbers are read independently of the process locale.
    const char* start = s_.c_str() + i_;
    const char* stop = s_.c_str() + s_.size();
    if (*start == '+') start++;  // jsoncpp accepts a leading '+'
    const auto r = std::from_chars(start, stop, v.num);
    if (r.ec != std::errc() || r.ptr == start) Fail("unexpected character");
    i_ = (size_t)(r.ptr - s_.c_str());
    v.kind = JVal::Num;
    return v;
  }

  std::string String() {
    std::string out;
    i_++;  // opening quote
    while (i_ < s_.size() && s_[i_] != '"') {
      char c = s_[i_++];
      if (c == '\\') {
        if (i_ >= s_.size()) Fail("unterminated string");
        const char e = s_[i_++];
        switch (e) {
          case 'n': c = '\n'; break;
          case 't': c = '\t'; break;
          case 'r': c = '\r'; break;
          case 'b': c = '\b'; break;
          case 'f': c = '\f'; break;
          case 'u': {  // \uXXXX: code points below 128 only (file names and keys)
            if (i_ + 4 > s_.size()) Fail("bad escape");
            const long cp = std::strtol(s_.substr(i_, 4).c_str(), nullptr, 16);
            i_ += 4;
            c = cp < 128 ? (char)cp : '?';
            break;
          }
          default: c = e;
        }
      }
      out.push_back(c);
    }
    if (i_ >= s_.size()) Fail("unterminated string");
    i_++;  // closing quote
    return out;
  }

  const std::string& s_;
  size_t i_ = 0;
};

// ReadJsonVec3f (main.cpp:24-27): components 0-2, a missing or non-numeric one is 0.
void vec3_of(const JVal* v, double out[3]) {
  for (int k = 0; k < 3; k++) {
    out[k] = 0.0;
    if (v && v->kind == JVal::Arr && (size_t)k < v->arr.size() && v->arr[k].kind == JVal::Num)
      out[k] = (double)(float)v->arr[k].num;  // asFloat
  }
}

// ---- OBJ -------------------------------------------------------------------
struct Corner {
  int v, n;  // 0-based indices, -1 for none
};

struct Mesh {
  std::vector<float> pos;  // corners of the triangles: 9 floats per triangle (scaled positions)
  std::vector<float> nrm;  // 9 floats per triangle
};

// Crossing-number point-in-polygon test (W. R. Franklin's published method),
// in the float arithmetic tinyobjloader uses.
bool pnpoly(int n, const float* xs, const float* ys, float tx, float ty) {
  bool c = false;
  for (int i = 0, j = n - 1; i < n; j = i++)
    if (((ys[i] > ty) != (ys[j] > ty)) && (tx < (xs[j] - xs[i]) * (ty - ys[i]) / (ys[j] - ys[i]) + xs[i])) c = !c;
  return c;
}

// Triangulation of one face as tinyobjloader 1.4 does it when asked to
// (dependencies/tiny_obj_loader/include/tiny_obj_loader.h:1105-1310): ear
// clipping in the plane of the two axes the first non-degenerate corner picks,
// from corner 0, a vertex inside a candidate ear rejecting it; a convex polygon
// becomes the fan from corner 0.  Corners with invalid position indices are
// dropped by the caller.
void triangulate(const std::vector<Corner>& face, const std::vector<float>& v, std::vector<Corner>& out) {
  const size_t np0 = face.size();
  if (np0 < 3) return;
  if (np0 == 3) {
    out.insert(out.end(), face.begin(), face.end());
    return;
  }
  auto P = [&](const Corner& c, int k) { return v[3 * (size_t)c.v + k]; };
  int axes[2] = {1, 2};
  for (size_t k = 0; k < np0; ++k) {
    const Corner& i0 = face[k % np0];
    const Corner& i1 = face[(k + 1) % np0];
    const Corner& i2 = face[(k + 2) % np0];
    const float e0x = P(i1, 0) - P(i0, 0), e0y = P(i1, 1) - P(i0, 1), e0z = P(i1, 2) - P(i0, 2);
    const float e1x = P(i2, 0) - P(i1, 0), e1y = P(i2, 1) - P(i1, 1), e1z = P(i2, 2) - P(i1, 2);
    const float cx = std::fabs(e0y * e1z - e0z * e1y);
    const float cy = std::fabs(e0z * e1x - e0x * e1z);
    const float cz = std::fabs(e0x * e1y - e0y * e1x);
    const float eps = std::numeric_limits<float>::epsilon();
    if (cx > eps || cy > eps || cz > eps) {
      if (!(cx > cy && cx > cz)) {
        axes[0] = 0;
        if (cz > cx && cz > cy) axes[1] = 1;
      }
      break;
    }
  }
  float area = 0.0f;
  for (size_t k = 0; k < np0; ++k) {
    const Corner& a = face[k % np0];
    const Corner& b = face[(k + 1) % np0];
    area += (P(a, axes[0]) * P(b, axes[1]) - P(a, axes[1]) * P(b, axes[0])) * 0.5f;
  }
  std::vector<Corner> rem = face;
  size_t guess = 0;
  size_t iters = rem.size(), prev = rem.size();
  while (rem.size() > 3 && iters > 0) {
    const size_t np = rem.size();
    if (guess >= np) guess -= np;
    if (prev != np) {
      prev = np;
      iters = np;
    } else {
      iters--;
    }
    Corner ind[3];
    float vx[3], vy[3];
    for (int k = 0; k < 3; k++) {
      ind[k] = rem[(guess + k) % np];
      vx[k] = P(ind[k], axes[0]);
      vy[k] = P(ind[k], axes[1]);
    }
    const float e0x = vx[1] - vx[0], e0y = vy[1] - vy[0];
    const float e1x = vx[2] - vx[1], e1y = vy[2] - vy[1];
    const float cross = e0x * e1y - e0y * e1x;
    if (cross * area < 0.0f) {  // a reflex corner
      guess += 1;
      continue;
    }
    bool overlap = false;
    for (size_t other = 3; other < np; ++other) {
      const Corner& o = rem[(guess + other) % np];
      if (pnpoly(3, vx, vy, P(o, axes[0]), P(o, axes[1]))) {
        overlap = true;
        break;
      }
    }
    if (overlap) {
      guess += 1;
      continue;
    }
    out.insert(out.end(), ind, ind + 3);  // an ear: emit it, drop its middle corner
    rem.erase(rem.begin() + (long)((guess + 1) % np));
  }
  if (rem.size() == 3) out.insert(out.end(), rem.begin(), rem.end());
}

int parse_index(const std::string& s, int count) {
  if (s.empty()) return -1;
  const long k = std::strtol(s.c_str(), nullptr, 10);
  if (k > 0) return (int)(k - 1);
  if (k < 0) return (int)(count + k);
  return -1;
}

Mesh load_obj(const std::string& path, const double scale[3]) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("scene file: cannot open mesh " + path);
  std::vector<float> v, vn;
  std::vector<std::vector<Corner>> faces;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    ss.imbue(std::locale::classic());  // numbers independent of the process locale
    std::string tag;
    if (!(ss >> tag)) continue;
    if (tag == "v" || tag == "vn") {
      double x, y, z;
      if (!(ss >> x >> y >> z)) continue;
      auto& dst = tag == "v" ? v : vn;
      dst.push_back((float)x);
      dst.push_back((float)y);
      dst.push_back((float)z);
    } else if (tag == "f") {
      std::vector<Corner> face;
      std::string tok;
      while (ss >> tok) {
        const size_t s1 = tok.find('/');
        const std::string a = tok.substr(0, s1);
        std::string c;
        if (s1 != std::string::npos) {
          const size_t s2 = tok.find('/', s1 + 1);
          if (s2 != std::string::npos) c = tok.substr(s2 + 1);
        }
        face.push_back(Corner{parse_index(a, (int)(v.size() / 3)), parse_index(c, (int)(vn.size() / 3))});
      }
      faces.push_back(std::move(face));
    }
  }
  Mesh m;
  const int nv = (int)(v.size() / 3), nn = (int)(vn.size() / 3);
  std::vector<Corner> tri;
  for (const auto& face : faces) {
    bool ok = face.size() >= 3;
    for (const Corner& c : face) ok = ok && c.v >= 0 && c.v < nv;
    if (!ok) continue;
    tri.clear();
    triangulate(face, v, tri);
    for (const Corner& c : tri) {
      for (int k = 0; k < 3; k++) m.pos.push_back((float)(v[3 * (size_t)c.v + k] * (float)scale[k]));
      if (c.n >= 0 && c.n < nn) {
        for (int k = 0; k < 3; k++) m.nrm.push_back(vn[3 * (size_t)c.n + k]);
      } else {
        m.nrm.push_back(1.0f);  // Mesh.h:48
        m.nrm.push_back(0.0f);
        m.nrm.push_back(0.0f);
      }
    }
  }
  return m;
}

bool file_exists(const std::string& p) {
  std::ifstream f(p);
  return (bool)f;
}

std::string dir_of(const std::string& p) {
  const size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

// The reference opens mesh paths relative to its working directory, a sibling
// of bin/data; tried: as given, next to the scene file, one and two folders up.
std::string resolve_mesh(const std::string& name, const std::string& scene_dir) {
  if (!name.empty() && name[0] == '/') return name;
  const std::string cands[4] = {name, scene_dir + "/" + name, scene_dir + "/../" + name,
                                scene_dir + "/../../_/" + name};
  for (const auto& c : cands)
    if (file_exists(c)) return c;
  throw std::runtime_error("scene file: mesh " + name + " not found (scene folder " + scene_dir + ")");
}

// glm::rotate(|a|, a / |a|) (Rodrigues' formula), row-major 3x3, in double.
void rotation(const double a[3], double R[9]) {
  const double th = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  for (int i = 0; i < 9; i++) R[i] = (i % 4 == 0) ? 1.0 : 0.0;
  if (th <= 1e-3) return;
  const double x = a[0] / th, y = a[1] / th, z = a[2] / th, c = std::cos(th), s = std::sin(th), t = 1.0 - c;
  const double M[9] = {c + t * x * x,     t * x * y - s * z, t * x * z + s * y,  //
                       t * x * y + s * z, c + t * y * y,     t * y * z - s * x,  //
                       t * x * z - s * y, t * y * z + s * x, c + t * z * z};
  for (int i = 0; i < 9; i++) R[i] = M[i];
}

}  // namespace
}  // namespace gi

struct gi_scene {
  std::vector<gi_mesh_object> objects;
  std::vector<gi_triangle> triangles;
  std::vector<std::string> mesh_names;
  int shadow_size = 1024;
};

using namespace gi;

extern "C" int gi_scene_load(const char* path, gi_scene** out) {
  GI_CHECK_ARG(path && out, "gi_scene_load: null argument");
  *out = nullptr;
  try {
    std::ifstream f(path);
    if (!f) return fail(GI_ERR_IO, std::string("gi_scene_load: cannot open ") + path);
    std::stringstream buf;
    buf << f.rdbuf();
    const std::string text = buf.str();
    const JVal root = JsonParser(text).Parse();
    std::unique_ptr<gi_scene> sc(new gi_scene());
    const JVal* rend = root.get("renderer");
    if (rend) {
      const JVal* ss = rend->get("shadowmapSize");
      if (ss && ss->kind == JVal::Arr && !ss->arr.empty() && ss->arr[0].kind == JVal::Num && ss->arr[0].num >= 1)
        sc->shadow_size = (int)ss->arr[0].num;
    }
    const JVal* scene = root.get("scene");
    const std::string sdir = dir_of(path);
    std::map<std::string, Mesh> meshes;
    const JVal* mlist = scene ? scene->get("meshes") : nullptr;
    if (mlist && mlist->kind == JVal::Arr) {
      for (const JVal& m : mlist->arr) {
        double scale[3];
        vec3_of(m.get("scale"), scale);
        meshes[m.get_string("name", "<unspecified>")] =
            load_obj(resolve_mesh(m.get_string("filename", "<unspecified>"), sdir), scale);
      }
    }
    const JVal* olist = scene ? scene->get("objects") : nullptr;
    int first = 0;
    if (olist && olist->kind == JVal::Arr) {
      for (const JVal& o : olist->arr) {
        const std::string name = o.get_string("mesh", "<unspecified>");
        auto it = meshes.find(name);
        if (it == meshes.end()) continue;  // Scene.h:95-99
        const Mesh& mesh = it->second;
        double angle[3], pos[3], albedo[3], emissive[3], R[9];
        vec3_of(o.get("angle"), angle);
        vec3_of(o.get("pos"), pos);
        vec3_of(o.get("albedoColor"), albedo);
        vec3_of(o.get("emissiveColor"), emissive);
        rotation(angle, R);
        const int count = (int)(mesh.pos.size() / 9);
        GI_CHECK_ARG((size_t)first + count <= (size_t)GI_MAX_TRIANGLES, "gi_scene_load: too many triangles");
        gi_mesh_object ob{};
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, big = 1.0;
        for (int t = 0; t < count; t++) {
          gi_triangle tr{};
          for (int c = 0; c < 3; c++) {
            const float* p = &mesh.pos[9 * (size_t)t + 3 * c];
            const float* n = &mesh.nrm[9 * (size_t)t + 3 * c];
            for (int r = 0; r < 3; r++) {
              const double w = R[3 * r] * p[0] + R[3 * r + 1] * p[1] + R[3 * r + 2] * p[2] + pos[r];
              tr.p[c][r] = (float)w;
              tr.n[c][r] = (float)(R[3 * r] * n[0] + R[3 * r + 1] * n[1] + R[3 * r + 2] * n[2]);
              lo[r] = std::fmin(lo[r], (double)tr.p[c][r]);
              hi[r] = std::fmax(hi[r], (double)tr.p[c][r]);
              big = std::fmax(big, std::fabs((double)tr.p[c][r]));
            }
          }
          sc->triangles.push_back(tr);
        }
        // Padded bounds: a ray that meets a triangle on the boundary still enters the box.
        const double pad = 1e-4 * big;
        for (int r = 0; r < 3; r++) {
          ob.lo[r] = count ? (float)(lo[r] - pad) : 0.0f;
          ob.hi[r] = count ? (float)(hi[r] + pad) : 0.0f;
        }
        ob.first = first;
        ob.count = count;
        for (int k = 0; k < 3; k++) {
          ob.albedo[k] = (float)albedo[k];
          ob.emissive[k] = (float)emissive[k];
        }
        ob.albedo[3] = ob.emissive[3] = 1.0f;
        sc->objects.push_back(ob);
        sc->mesh_names.push_back(name);
        first += count;
      }
    }
    GI_CHECK_ARG(sc->objects.size() <= (size_t)GI_MAX_MESH_OBJECTS, "gi_scene_load: too many objects");
    *out = sc.release();
    return GI_OK;
  } catch (const std::exception& e) {
    return fail(GI_ERR_IO, e.what());
  }
}

extern "C" int gi_scene_info(const gi_scene* s, int* num_objects, int* num_triangles, int* shadow_size) {
  GI_CHECK_ARG(s && num_objects && num_triangles && shadow_size, "gi_scene_info: null argument");
  *num_objects = (int)s->objects.size();
  *num_triangles = (int)s->triangles.size();
  *shadow_size = s->shadow_size;
  return GI_OK;
}

extern "C" int gi_scene_copy(const gi_scene* s, gi_mesh_object* objects, gi_triangle* triangles) {
  GI_CHECK_ARG(s && (objects || s->objects.empty()) && (triangles || s->triangles.empty()),
               "gi_scene_copy: null argument");
  if (!s->objects.empty()) std::memcpy(objects, s->objects.data(), s->objects.size() * sizeof(gi_mesh_object));
  if (!s->triangles.empty()) std::memcpy(triangles, s->triangles.data(), s->triangles.size() * sizeof(gi_triangle));
  return GI_OK;
}

extern "C" const char* gi_scene_object_mesh(const gi_scene* s, int i) {
  if (!s || i < 0 || (size_t)i >= s->mesh_names.size()) return nullptr;
  return s->mesh_names[(size_t)i].c_str();
}

extern "C" int gi_scene_destroy(gi_scene* s) {
  delete s;
  return GI_OK;
}
