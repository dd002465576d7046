// Scene front end: the reference's scene text format (SceneEnv::Load,
// scene_env.h:357-2160) and its OBJ meshes (Obj::Load, ObjLoader.cpp:40-500)
// read into the plain structs that pr_scene_upload and pr_render take.
//
// The reader follows the reference's line rules: an upper-case setting's
// keyword on one line and its value on the next; one '#' comment line
// skipped before a keyword (getLine, scene_env.h:141-149) and '#' lines
// skipped inside blocks; OBJECT, BLACKHOLE and WORMHOLE blocks end at an
// empty line.
// Every value the reference reads through its expression evaluator is read
// through the same rules here (scene_expr.h: VAR variables, arithmetic,
// functions); values it reads with sscanf are read with sscanf.
//
// It reads the keywords of the features this library renders (spheres,
// uvplanes, disks, OBJ meshes; diffuse / specular / glass / Ward / Phong /
// subsurface materials; rotation / translate / scale of spheres and meshes;
// the global medium; TARGET_POS and CAMERA_MATRIX; the black hole with its
// background and accretion-disk textures; the wormhole with its two
// backgrounds; spot, parallel and infinity lights; textures, IBL images and
// bump maps).  A keyword that changes the image through a feature this
// library does not render (transformed uvplanes and disks, lens, MLT / ERPT,
// dispersion ...) is refused with an error naming the line, so
// that no scene renders silently different; settings that do not change
// the image (THREAD, OUTPUT, ...) are skipped.  The reference's overrides
// of settings by environment variables (SAMPLING, IMAGE_X, USE_BSSRDF ...)
// are not applied; a value written as %NAME% is read from the environment,
// as the reference reads it.  Textures must be uncompressed 24- or 32-bit
// BMP files.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <initializer_list>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/prender_gpu.h"
#include "scene_build.h"
#include "scene_expr.h"

struct pr_scene_file {
  std::string warnings;
  std::vector<pr_material> mats;
  std::vector<pr_entity> ents;
  std::vector<std::vector<float>> verts;
  std::vector<std::vector<int32_t>> faces;
  std::vector<std::vector<float>> fnormals;  // empty: the loader's rule at upload
  // per mesh: vertex normals with their face ids (empty: derived at upload)
  // and texture coordinates with theirs (empty: none)
  std::vector<std::vector<float>> vnormals, uvs;
  std::vector<std::vector<int32_t>> face_vn, face_uv;
  // per mesh: OBJ materials, their map_Kd images, each face's material
  std::vector<std::vector<pr_obj_material>> omats;
  std::vector<std::vector<std::vector<uint8_t>>> omat_tex;
  std::vector<std::vector<int32_t>> fmat;
  std::vector<pr_mesh> meshes;
  std::vector<uint8_t> bg_tex, disk_tex, worm_tex[2];
  // per material: texture / IBL images (pointers set when the desc is made)
  std::vector<std::vector<uint8_t>> tex8, ibl8, bump8;
  std::vector<std::vector<float>> iblf;
  pr_scene_desc desc;
  pr_camera cam;
  pr_render_params prm;
  double gamma_offset = 0.0;
};

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kRad = kPi / 180.0;  // PS_RAD (constant.h:31)
constexpr double kEps = 1.0e-6;       // PS_EPS (constant.h:36)

struct LoadError {
  std::string what;
};

[[noreturn]] void fail(const std::string& s) { throw LoadError{s}; }

std::string trim_eol(const std::string& s) {
  size_t e = s.size();
  while (e > 0 && (s[e - 1] == '\n' || s[e - 1] == '\r')) e--;
  return s.substr(0, e);
}

std::vector<std::string> tokens(const std::string& s) {
  std::vector<std::string> t;
  std::istringstream is(s);
  std::string w;
  while (is >> w) t.push_back(w);
  return t;
}

// the text after a line's first blank (what sscanf*fs evaluates)
std::string after_key(const std::string& line) {
  const size_t p = line.find(' ');
  return p == std::string::npos ? std::string() : line.substr(p + 1);
}

bool starts(const std::string& s, const char* p) { return s.compare(0, std::strlen(p), p) == 0; }

bool among(const std::string& k, std::initializer_list<const char*> kw) {
  for (const char* s : kw)
    if (k == s) return true;
  return false;
}

class Reader {
 public:
  explicit Reader(const std::string& path) : f_(std::fopen(path.c_str(), "r")) {
    if (!f_) fail("cannot open scene file " + path);
  }
  ~Reader() {
    if (f_) std::fclose(f_);
  }
  Reader(const Reader&) = delete;
  Reader& operator=(const Reader&) = delete;
  // getLine: one '#' line is skipped
  bool get(std::string& out) {
    if (!raw(out)) return false;
    if (!out.empty() && out[0] == '#') return raw(out);
    return true;
  }
  // one line as fgets reads it inside a block
  bool raw(std::string& out) {
    char buf[4096];
    if (!std::fgets(buf, sizeof buf, f_)) return false;
    out = trim_eol(buf);
    line_++;
    return true;
  }
  std::string value(const std::string& key) {
    std::string v;
    if (!get(v)) fail("missing value after " + key);
    return v;
  }
  int line() const { return line_; }

 private:
  FILE* f_;
  int line_ = 0;
};

// Numbers: the expression forms and the sscanf forms of the reference
struct Numbers {
  pr::ExprReader ex;
  double one(const std::string& s) {
    try {
      return ex.one(s);
    } catch (const pr::ExprError& e) {
      fail(e.what());
    }
  }
  std::vector<double> many(const std::string& s, int n) {
    try {
      return ex.many(s, n);
    } catch (const pr::ExprError& e) {
      fail(e.what());
    }
  }
  int integer(const std::string& s) { return (int)one(s); }  // atoi: truncation toward zero
};

// sscanf with one %d or %lf: the variable keeps its value when nothing matches
template <typename T>
void scan(const std::string& s, const char* fmt, T& v) {
  T t = v;
  if (std::sscanf(s.c_str(), fmt, &t) == 1) v = t;
}

std::string dir_of(const std::string& path) {
  const size_t p = path.find_last_of('/');
  return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

bool readable(const std::string& p) {
  if (FILE* f = std::fopen(p.c_str(), "rb")) {
    std::fclose(f);
    return true;
  }
  return false;
}

// a file named in the scene: as given (the reference opens it from the
// working directory first), else beside the scene file
std::string resolve(const std::string& name, const std::string& scene_dir) {
  if (readable(name)) return name;
  if (readable(scene_dir + name)) return scene_dir + name;
  fail("cannot open " + name);
}

// An uncompressed 24- or 32-bit BMP as RGB8 (channels 3) or RGBA8 (4) rows
// in the order Bitmap::cell(y, x) reads them (bitmap.h:187-190: row H-1-y
// of the top-down image, so the picture's bottom row comes first).  A
// 24-bit image has alpha 255 (BitMap::Read, bitmap.cpp:116-123); a 32-bit
// image whose alpha bytes are all zero reads as opaque, as the image
// decoder the reference uses treats it.
void read_bmp(const std::string& path, int channels, std::vector<uint8_t>& out, int& w, int& h) {
  std::ifstream f(path, std::ios::binary);
  std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  auto u32 = [&](size_t o) {
    return (uint32_t)d[o] | ((uint32_t)d[o + 1] << 8) | ((uint32_t)d[o + 2] << 16) | ((uint32_t)d[o + 3] << 24);
  };
  auto u16 = [&](size_t o) { return (uint32_t)d[o] | ((uint32_t)d[o + 1] << 8); };
  if (d.size() < 54 || d[0] != 'B' || d[1] != 'M') fail("not a BMP file: " + path + " (textures must be BMP)");
  const uint32_t off = u32(10);
  const int32_t W = (int32_t)u32(18), H = (int32_t)u32(22);
  const uint32_t bpp = u16(28), comp = u32(30);
  bool ok = (bpp == 24 || bpp == 32) && comp == 0;
  if (bpp == 32 && comp == 3 && d.size() >= 66)  // bit fields: only the plain BGRA layout
    ok = u32(54) == 0x00FF0000u && u32(58) == 0x0000FF00u && u32(62) == 0x000000FFu;
  if (!ok || W <= 0 || W > (1 << 16) || H == 0 || H > (1 << 16) || H < -(1 << 16))
    fail("unsupported BMP (uncompressed 24- or 32-bit only): " + path);
  w = W;
  h = H < 0 ? -H : H;
  const size_t bytes = bpp / 8;
  const size_t row = ((size_t)W * bytes + 3) & ~(size_t)3;
  if (d.size() < off + row * (size_t)h) fail("truncated BMP: " + path);
  out.assign((size_t)w * h * channels, 255);
  bool any_alpha = false;
  for (int y = 0; y < h; y++) {
    // positive height: rows stored bottom-up, so stored row y is cell row y
    const int fy = H > 0 ? y : h - 1 - y;
    const uint8_t* r = d.data() + off + row * (size_t)fy;
    for (int x = 0; x < w; x++) {
      const uint8_t* px = r + (size_t)x * bytes;
      uint8_t* o = out.data() + ((size_t)y * w + x) * channels;
      o[0] = px[2];
      o[1] = px[1];
      o[2] = px[0];
      if (channels == 4 && bpp == 32) {
        o[3] = px[3];
        any_alpha |= px[3] != 0;
      }
    }
  }
  if (channels == 4 && bpp == 32 && !any_alpha)
    for (size_t i = 3; i < out.size(); i += 4) out[i] = 255;
}

// HDRImage::load_unsafe (hdr.h:82-210): a Radiance file with the
// '#?RADIANCE' line and '-Y H +X W', new-style run-length scanlines (reading
// stops at the first scanline without the 2 2 marker; rows not read stay
// zero), each value byte * 2^(e - 128) / 256 (e = 0 included), file row y
// stored as image row H - 1 - y; out: float RGB in IBL_Color(i, j) order
void read_hdr(const std::string& path, std::vector<float>& out, int& w, int& h) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail("cannot open " + path);
  std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t p = 0;
  bool valid = false;
  auto line = [&]() {
    std::string l;
    while (p < d.size() && d[p] != '\n') l += (char)d[p++];
    if (p < d.size()) p++;
    return l;
  };
  for (;;) {
    if (p >= d.size()) fail("truncated HDR header: " + path);
    const std::string l = line();
    if (l == "#?RADIANCE") valid = true;
    if (l.empty()) break;
  }
  if (!valid) fail("not a Radiance HDR file: " + path);
  char a[64] = {0}, b[64] = {0};
  int H = 0, W = 0;
  const std::string res = line();
  if (std::sscanf(res.c_str(), "%63s %d %63s %d", a, &H, b, &W) != 4 || std::string(a) != "-Y" ||
      std::string(b) != "+X" || W <= 0 || H <= 0 || W > (1 << 16) || H > (1 << 16))
    fail("unsupported HDR orientation or size (only '-Y H +X W'): " + path);
  w = W;
  h = H;
  std::vector<uint8_t> tmp((size_t)W * H * 4, 0);
  for (int y = 0; y < H; y++) {
    if (p + 4 > d.size() || d[p] != 2 || d[p + 1] != 2) break;
    const int lw = (d[p + 2] << 8) + d[p + 3];
    p += 4;
    int x = 0, c = 0;
    for (;;) {
      if (x >= lw) {
        c++;
        x = 0;
        if (c == 4) break;
      }
      if (p >= d.size()) fail("truncated HDR data: " + path);
      const int info = d[p++];
      const int n = info <= 128 ? info : info - 128;
      for (int k = 0; k < n; k++) {
        if (x >= W) fail("HDR scanline longer than the image: " + path);
        if (info <= 128 && p >= d.size()) fail("truncated HDR data: " + path);
        const uint8_t v = info <= 128 ? d[p++] : d[p];
        tmp[((size_t)y * W + x) * 4 + c] = v;
        x++;
      }
      if (info > 128) p++;
    }
  }
  out.assign((size_t)W * H * 3, 0.0f);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const uint8_t* t = tmp.data() + ((size_t)y * W + x) * 4;
      const double sc = std::pow(2.0, (double)t[3] - 128.0) / 256.0;
      for (int c = 0; c < 3; c++) out[((size_t)(H - 1 - y) * W + x) * 3 + c] = (float)(t[c] * sc);
    }
}

struct ObjMesh {
  std::vector<pr_obj_material> mats;         // newmtl entries (mtllib)
  std::vector<std::string> mat_names;
  std::vector<std::vector<uint8_t>> mat_tex;  // map_Kd images (RGB)
  std::vector<int32_t> fmat;                  // per triangle: usemtl index, -1 none
  std::vector<float> v;      // 3 per vertex
  std::vector<float> vn;     // 3 per vertex normal
  std::vector<float> vt;     // 2 per texture coordinate
  std::vector<int32_t> f;    // 3 per triangle, 0-based
  std::vector<int32_t> nid;  // 3 per triangle: vertex-normal ids (0 where the face gives none)
  std::vector<int32_t> tid;  // 3 per triangle: texture-coordinate ids (empty without vt lines)
};

// Obj::Load (ObjLoader.cpp:125-470): 'v', 'vn' and 'vt' lines as floats;
// faces in the reference's order of attempts (v/vt/vn, v//vn, v/vt, v; four
// vertices before three), a quad a b c d split into (a, b, c) and (c, d, a)
// with its normal and texture ids alike; ids a face does not give are 0.
// Vertex colours (a last 'v' line with six or more numbers makes the whole
// mesh take them, ObjLoader.cpp:199-228) are refused.
// Obj::LoadMTLFile (ObjLoader.cpp:704-900): lines after leading blanks,
// dispatched on the first character as the reference does (any line that
// starts with 'n' opens a material; K a/d/s, d, Tr, Ni, Ns, map_Kd,
// map_Bump and the '#' extensions); a map_Kd name is tried as given, then
// beside the MTL file (Polygon::LoadTexture, polygon.h:971-1030).
void read_mtl(const std::string& file, ObjMesh& m) {
  std::ifstream f(file);
  if (!f) return;
  std::string line;
  pr_obj_material* cur = nullptr;
  while (std::getline(f, line)) {
    size_t b = 0;
    while (b < line.size() && (line[b] == ' ' || line[b] == '\t')) b++;
    const std::string s = trim_eol(line.substr(b));
    if (s.empty()) continue;
    const char* c = s.c_str();
    float x = 0, y = 0, z = 0;
    switch (c[0]) {
      case 'n': {
        pr_obj_material o;
        memset(&o, 0, sizeof(o));
        o.alpha = -1.0;
        o.shininess = 5.0;
        o.reflection = -1;
        o.repeat = 1;
        m.mats.push_back(o);
        char name[128] = {0};
        std::sscanf(c, "newmtl %127s", name);
        m.mat_names.push_back(name);
        m.mat_tex.emplace_back();
        cur = &m.mats.back();
        break;
      }
      case 'K':
        if (!cur) break;
        if (c[1] == 'd') {
          const int n = std::sscanf(c, "Kd %f %f %f", &x, &y, &z);
          const double v3[3] = {x, y, z};
          for (int i = 0; i < n; i++) cur->diffuse[i] = v3[i];
        } else if (c[1] == 's') {
          const int n = std::sscanf(c, "Ks %f %f %f", &x, &y, &z);
          const double v3[3] = {x, y, z};
          for (int i = 0; i < n; i++) cur->specular[i] = v3[i];
        }
        break;
      case 'd':
        if (cur && std::sscanf(c, "d %f", &x) == 1) cur->alpha = x;
        break;
      case 'T':
        if (cur && c[1] == 'r' && std::sscanf(c, "Tr %f", &x) == 1) cur->alpha = std::max(0.0, 1.0 - x);
        break;
      case 'N':
        if (cur && c[1] == 'i' && std::sscanf(c, "Ni %f", &x) == 1) cur->refraction_index = x;
        if (cur && c[1] == 's' && std::sscanf(c, "Ns %f", &x) == 1) cur->shininess = x;
        break;
      case 'm':
        if (cur && starts(s, "map_Kd") && s.size() > 7) {
          std::string name = s.substr(7);
          const std::string p = readable(name) ? name : dir_of(file) + name;
          int w = 0, h = 0;
          std::vector<uint8_t> rgba;
          read_bmp(p, 4, rgba, w, h);
          for (size_t q = 0; q < (size_t)w * h; q++)
            if (rgba[4 * q + 3] != 255) fail("a map_Kd texture with transparent texels is not rendered here: " + p);
          std::vector<uint8_t>& t = m.mat_tex.back();
          t.resize(3 * (size_t)w * h);
          for (size_t q = 0; q < (size_t)w * h; q++)
            for (int a = 0; a < 3; a++) t[3 * q + a] = rgba[4 * q + a];
          cur->texture_width = w;
          cur->texture_height = h;
        }
        break;
      case '#': {
        if (!cur) break;
        int iv = 0;
        if (starts(s, "#SMOOTH ") && std::sscanf(c, "#SMOOTH %d", &iv) >= 0) cur->smooth = iv ? 1 : 2;
        if (starts(s, "#REFLECTION ")) {
          std::sscanf(c, "#REFLECTION %d", &cur->reflection);
          if (cur->reflection == 0 || cur->reflection == 1) cur->roughness = 0.0;
          if (cur->reflection == 2 && (float)cur->refraction_index == 0.0f) cur->refraction_index = 1.5;
        }
        if (starts(s, "#EMISSION ")) {
          const int n = std::sscanf(c, "#EMISSION %f %f %f", &x, &y, &z);
          const double v3[3] = {x, y, z};
          for (int i = 0; i < n; i++) cur->emission[i] = v3[i];
        }
        if (starts(s, "#COLOR ")) {
          const int n = std::sscanf(c, "#COLOR %f %f %f", &x, &y, &z);
          const double v3[3] = {x, y, z};
          for (int i = 0; i < n; i++) cur->diffuse[i] = v3[i];
        }
        if (starts(s, "#WARD ")) {
          const int n = std::sscanf(c, "#WARD %f %f", &x, &y);
          if (n >= 1) cur->ward[0] = x;
          if (n >= 2) cur->ward[1] = y;
        }
        if (starts(s, "#SPECULAR ")) {
          const int n = std::sscanf(c, "#SPECULAR %f %f %f", &x, &y, &z);
          const double v3[3] = {x, y, z};
          for (int i = 0; i < n; i++) cur->specular[i] = v3[i];
        }
        if (starts(s, "#ROUGHNESS ") && std::sscanf(c, "#ROUGHNESS %f", &x) == 1) cur->roughness = x;
        if (starts(s, "#REPEAT ")) std::sscanf(c, "#REPEAT %d", &cur->repeat);
        break;
      }
      default:
        break;
    }
  }
}

void read_obj(const std::string& path, ObjMesh& m) {
  std::ifstream f(path);
  if (!f) fail("cannot open " + path);
  std::string line, mtllib;
  bool vertex_colour = false;
  int32_t cur_mat = -1;
  while (std::getline(f, line)) {
    size_t b = 0;
    while (b < line.size() && (line[b] == ' ' || line[b] == '\t')) b++;
    const std::string s = line.substr(b);
    const char* c = s.c_str();
    if (starts(s, "mtllib ")) {  // the file as given, else beside the OBJ (ObjLoader.cpp:137-157)
      mtllib = trim_eol(s.substr(7));
      read_mtl(readable(mtllib) ? mtllib : dir_of(path) + mtllib, m);
    } else if (starts(s, "usemtl ")) {  // the last material of that name, case-insensitive (:159-180)
      const std::string name = trim_eol(s.substr(7));
      cur_mat = -1;
      for (size_t i = 0; i < m.mat_names.size(); i++) {
        const std::string& a = m.mat_names[i];
        bool eq = a.size() == name.size();
        for (size_t q = 0; eq && q < a.size(); q++) eq = std::tolower((unsigned char)a[q]) == std::tolower((unsigned char)name[q]);
        if (eq) cur_mat = (int32_t)i;
      }
    } else if (s.size() > 1 && c[0] == 'v' && c[1] == 'n') {
      float x = 0, y = 0, z = 0;
      std::sscanf(c, "%*s %f %f %f", &x, &y, &z);
      m.vn.insert(m.vn.end(), {x, y, z});
    } else if (s.size() > 1 && c[0] == 'v' && c[1] == 't') {
      float x = 0, y = 0;
      std::sscanf(c, "%*s %f %f", &x, &y);
      m.vt.insert(m.vt.end(), {x, y});
    } else if (s.size() > 1 && c[0] == 'v' && c[1] == ' ') {
      float x = 0, y = 0, z = 0, cr[3];
      vertex_colour = std::sscanf(c, "%*s %f %f %f %f %f %f", &x, &y, &z, &cr[0], &cr[1], &cr[2]) == 6;
      m.v.insert(m.v.end(), {x, y, z});
    } else if (s.size() > 1 && c[0] == 'f' && c[1] == ' ') {
      const char* p = c + 2;
      int a[4], t[4], n[4];
      bool has_n = false, has_t = false;
      int k = 0;
      if (std::sscanf(p, "%d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d", &a[0], &t[0], &n[0], &a[1], &t[1], &n[1], &a[2], &t[2],
                      &n[2], &a[3], &t[3], &n[3]) == 12) {
        k = 4, has_n = has_t = true;
      } else if (std::sscanf(p, "%d/%d/%d %d/%d/%d %d/%d/%d", &a[0], &t[0], &n[0], &a[1], &t[1], &n[1], &a[2], &t[2],
                             &n[2]) == 9) {
        k = 3, has_n = has_t = true;
      } else if (std::sscanf(p, "%d//%d %d//%d %d//%d %d//%d", &a[0], &n[0], &a[1], &n[1], &a[2], &n[2], &a[3],
                             &n[3]) == 8) {
        k = 4, has_n = true;
      } else if (std::sscanf(p, "%d//%d %d//%d %d//%d", &a[0], &n[0], &a[1], &n[1], &a[2], &n[2]) == 6) {
        k = 3, has_n = true;
      } else if (std::sscanf(p, "%d/%d %d/%d %d/%d %d/%d", &a[0], &t[0], &a[1], &t[1], &a[2], &t[2], &a[3], &t[3]) ==
                 8) {
        k = 4, has_t = true;
      } else if (std::sscanf(p, "%d/%d %d/%d %d/%d", &a[0], &t[0], &a[1], &t[1], &a[2], &t[2]) == 6) {
        k = 3, has_t = true;
      } else if (std::sscanf(p, "%d %d %d %d", &a[0], &a[1], &a[2], &a[3]) == 4) {
        k = 4;
      } else if (std::sscanf(p, "%d %d %d", &a[0], &a[1], &a[2]) == 3) {
        k = 3;
      } else {
        fail("face line not read: " + path + ": " + line);
      }
      if (!has_n)
        for (int i = 0; i < 4; i++) n[i] = 1;  // no ids: the reference's zero-initialised norm_id
      if (!has_t)
        for (int i = 0; i < 4; i++) t[i] = 1;  // and texture_id
      const int tri[2][3] = {{0, 1, 2}, {2, 3, 0}};
      for (int q = 0; q < (k == 4 ? 2 : 1); q++)
        for (int j = 0; j < 3; j++) {
          m.f.push_back(a[tri[q][j]] - 1);
          m.nid.push_back(n[tri[q][j]] - 1);
          m.tid.push_back(t[tri[q][j]] - 1);
        }
      for (int q = 0; q < (k == 4 ? 2 : 1); q++) m.fmat.push_back(cur_mat);
    }
  }
  const int64_t nv = (int64_t)(m.v.size() / 3), nn = (int64_t)(m.vn.size() / 3);
  for (int32_t i : m.f)
    if (i < 0 || i >= nv) fail("face index outside the vertices in " + path);
  if (nn > 0)
    for (int32_t i : m.nid)
      if (i < 0 || i >= nn) fail("vertex-normal index outside the normals in " + path);
  const int64_t nt = (int64_t)(m.vt.size() / 2);
  if (nt == 0) m.tid.clear();  // no vt lines: no texture ids (ObjLoader.cpp:474-478)
  for (int32_t i : m.tid)
    if (i < 0 || i >= nt) fail("texture-coordinate index outside the vt lines in " + path);
  if (vertex_colour) fail("OBJ vertex colours are not rendered here: " + path);
  if (m.f.empty()) fail("no faces in " + path);
  if (m.mats.empty()) m.fmat.clear();
}

// Obj::CalcNormalVector with vertex normals (ObjLoader.cpp:617-641): the
// face normal is the normalised mean of its three vertex normals
void face_normals_from_vn(const ObjMesh& m, std::vector<float>& out) {
  const size_t nf = m.f.size() / 3;
  out.resize(3 * nf);
  for (size_t i = 0; i < nf; i++) {
    float c[3];
    for (int a = 0; a < 3; a++) {
      const float s = (m.vn[3 * (size_t)m.nid[3 * i] + a] + m.vn[3 * (size_t)m.nid[3 * i + 1] + a]) +
                      m.vn[3 * (size_t)m.nid[3 * i + 2] + a];
      c[a] = (float)(s / 3.0);
    }
    double ln = (double)((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
    if (ln > 1.0e-16) {
      ln = std::sqrt(ln);
      for (int a = 0; a < 3; a++) c[a] = (float)(c[a] / ln);
    }
    for (int a = 0; a < 3; a++) out[3 * i + a] = c[a];
  }
}

// ---- transforms (matrix.h): row-major 4x4, points as row vectors ----
struct M4 {
  double a[16];
  double& operator()(int i, int j) { return a[4 * i + j]; }
  double operator()(int i, int j) const { return a[4 * i + j]; }
  static M4 identity() {
    M4 m;
    for (int i = 0; i < 16; i++) m.a[i] = (i % 5 == 0) ? 1.0 : 0.0;
    return m;
  }
};

// the three elementary rotations, the translation and the scale (matrix.h:120-172)
M4 rotation(int axis, double angle) {
  M4 m = M4::identity();
  const int i = axis == 0 ? 1 : 0, j = axis == 2 ? 1 : 2;
  m(i, i) = m(j, j) = std::cos(angle);
  if (axis == 1) {  // RotationY puts the sine below the diagonal
    m(j, i) = std::sin(angle);
    m(i, j) = -m(j, i);
  } else {
    m(i, j) = std::sin(angle);
    m(j, i) = -m(i, j);
  }
  return m;
}

M4 translation(double x, double y, double z) {
  M4 m = M4::identity();
  m(3, 0) = x;
  m(3, 1) = y;
  m(3, 2) = z;
  return m;
}

M4 scaling(double x, double y, double z) {
  M4 m = M4::identity();
  m(0, 0) = x;
  m(1, 1) = y;
  m(2, 2) = z;
  return m;
}

// point times matrix, with the translation row (matrix.h:399-407)
void apply(const M4& m, const double v[3], double o[3]) {
  for (int j = 0; j < 3; j++) o[j] = v[0] * m(0, j) + v[1] * m(1, j) + v[2] * m(2, j) + m(3, j);
}

// the inverse by cofactors over the determinant's reciprocal (the
// reference's InvertMatrix_, matrix.h:255-385; the cofactor expansion
// published with the Mesa GLU library), then transposed: the matrix
// that carries normals (vector_coordinate_transformation, matrix.h:204-208)
M4 normal_matrix(const M4& M) {
  const double* A = M.a;
  double inv[16];
  inv[0] = A[5] * A[10] * A[15] - A[5] * A[11] * A[14] - A[9] * A[6] * A[15] + A[9] * A[7] * A[14] +
           A[13] * A[6] * A[11] - A[13] * A[7] * A[10];
  inv[4] = -A[4] * A[10] * A[15] + A[4] * A[11] * A[14] + A[8] * A[6] * A[15] - A[8] * A[7] * A[14] -
           A[12] * A[6] * A[11] + A[12] * A[7] * A[10];
  inv[8] = A[4] * A[9] * A[15] - A[4] * A[11] * A[13] - A[8] * A[5] * A[15] + A[8] * A[7] * A[13] +
           A[12] * A[5] * A[11] - A[12] * A[7] * A[9];
  inv[12] = -A[4] * A[9] * A[14] + A[4] * A[10] * A[13] + A[8] * A[5] * A[14] - A[8] * A[6] * A[13] -
            A[12] * A[5] * A[10] + A[12] * A[6] * A[9];
  inv[1] = -A[1] * A[10] * A[15] + A[1] * A[11] * A[14] + A[9] * A[2] * A[15] - A[9] * A[3] * A[14] -
           A[13] * A[2] * A[11] + A[13] * A[3] * A[10];
  inv[5] = A[0] * A[10] * A[15] - A[0] * A[11] * A[14] - A[8] * A[2] * A[15] + A[8] * A[3] * A[14] +
           A[12] * A[2] * A[11] - A[12] * A[3] * A[10];
  inv[9] = -A[0] * A[9] * A[15] + A[0] * A[11] * A[13] + A[8] * A[1] * A[15] - A[8] * A[3] * A[13] -
           A[12] * A[1] * A[11] + A[12] * A[3] * A[9];
  inv[13] = A[0] * A[9] * A[14] - A[0] * A[10] * A[13] - A[8] * A[1] * A[14] + A[8] * A[2] * A[13] +
            A[12] * A[1] * A[10] - A[12] * A[2] * A[9];
  inv[2] = A[1] * A[6] * A[15] - A[1] * A[7] * A[14] - A[5] * A[2] * A[15] + A[5] * A[3] * A[14] +
           A[13] * A[2] * A[7] - A[13] * A[3] * A[6];
  inv[6] = -A[0] * A[6] * A[15] + A[0] * A[7] * A[14] + A[4] * A[2] * A[15] - A[4] * A[3] * A[14] -
           A[12] * A[2] * A[7] + A[12] * A[3] * A[6];
  inv[10] = A[0] * A[5] * A[15] - A[0] * A[7] * A[13] - A[4] * A[1] * A[15] + A[4] * A[3] * A[13] +
            A[12] * A[1] * A[7] - A[12] * A[3] * A[5];
  inv[14] = -A[0] * A[5] * A[14] + A[0] * A[6] * A[13] + A[4] * A[1] * A[14] - A[4] * A[2] * A[13] -
            A[12] * A[1] * A[6] + A[12] * A[2] * A[5];
  inv[3] = -A[1] * A[6] * A[11] + A[1] * A[7] * A[10] + A[5] * A[2] * A[11] - A[5] * A[3] * A[10] -
           A[9] * A[2] * A[7] + A[9] * A[3] * A[6];
  inv[7] = A[0] * A[6] * A[11] - A[0] * A[7] * A[10] - A[4] * A[2] * A[11] + A[4] * A[3] * A[10] +
           A[8] * A[2] * A[7] - A[8] * A[3] * A[6];
  inv[11] = -A[0] * A[5] * A[11] + A[0] * A[7] * A[9] + A[4] * A[1] * A[11] - A[4] * A[3] * A[9] -
            A[8] * A[1] * A[7] + A[8] * A[3] * A[5];
  inv[15] = A[0] * A[5] * A[10] - A[0] * A[6] * A[9] - A[4] * A[1] * A[10] + A[4] * A[2] * A[9] +
            A[8] * A[1] * A[6] - A[8] * A[2] * A[5];
  double det = A[0] * inv[0] + A[1] * inv[4] + A[2] * inv[8] + A[3] * inv[12];
  if (det == 0.0) fail("a singular transform (scale 0) cannot carry normals");
  det = 1.0 / det;
  M4 g;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) g(i, j) = inv[4 * j + i] * det;
  return g;
}

// Polygon::MatrixTransformation (polygon.h:749-772): each matrix in turn
// moves the float vertices (through double) and carries the float face
// normals, renormalised
void transform_mesh(const std::vector<M4>& ms, std::vector<float>& v, std::vector<float>& fn, std::vector<float>& vn) {
  for (const M4& m : ms) {
    for (size_t i = 0; i < v.size(); i += 3) {
      const double p[3] = {v[i], v[i + 1], v[i + 2]};
      double o[3];
      apply(m, p, o);
      for (int a = 0; a < 3; a++) v[i + a] = (float)o[a];
    }
    const M4 g = normal_matrix(m);
    for (std::vector<float>* nn : {&fn, &vn})  // face normals, then vertex normals (polygon.h:749-783)
      for (size_t i = 0; i < nn->size(); i += 3) {
        float* x = nn->data() + i;
        const double n[3] = {x[0], x[1], x[2]};
        double o[3];
        apply(g, n, o);
        const double inv = 1.0 / std::sqrt((o[0] * o[0] + o[2] * o[2]) + o[1] * o[1]);
        for (int a = 0; a < 3; a++) x[a] = (float)(o[a] * inv);
      }
  }
}

pr_medium default_medium() {
  pr_medium m;
  memset(&m, 0, sizeof(m));
  m.scale = 1.0;
  m.r_max = 1.0;
  m.level = -1;
  m.use_bssrdf = 1;
  return m;
}

// Material::Material (material.h:62-97).  The reference leaves the Ward
// roughness and the Phong exponent unset until a ward_brdf / phong_brdf
// line; they start at 0.1, 0.1 and 1 here.
pr_material default_material() {
  pr_material m;
  memset(&m, 0, sizeof(m));
  m.type = PR_MAT_DIFFUSE;
  m.refractive_index = 1.5;
  m.r_refractive_index = 1.0;
  m.medium = default_medium();
  m.ward_alpha[0] = m.ward_alpha[1] = 0.1;
  m.phong_exponent = 1.0;
  m.ibl_coef = 1.0;  // material.h:84-89
  m.repeat = 1;
  return m;
}

bool is_sss(int t) { return t == PR_MAT_SSS_REFRACTION || t == PR_MAT_SSS_DIFFUSE || t == PR_MAT_SSS_WARD; }

struct BlackHole {
  bool exists = false, pos_set = false;
  double pos[3] = {0, 0, 0}, dist = 10000.0, a = 0.0, steps = 10000.0, rdisk = 0.0;
  double map_coef[4] = {1.0, 0.0, 1.0, 0.0}, tex_coef = 1.0;
  int init_cond = 0;
  std::string bg_texture, disk_texture;
};

// the WORMHOLE block's settings with SceneEnv::Default's values
// (scene_env.h:262-300, :767-856)
struct Worm {
  bool exists = false, pos_set = false;
  double in[3] = {0, 0, 0}, out[3] = {0, 0, 0};
  double rho = 1.3, a = 0.5, w = 0.05, sign = 0.0, dist = 10000.0;
  double map_coef[2][4] = {{1.0, 0.0, 1.0, 0.0}, {1.0, 0.0, 1.0, 0.0}}, coef[2] = {1.0, 1.0};
  std::string texture[2];
};

class Loader {
 public:
  Loader(pr_scene_file& S, const std::string& path) : S_(S), path_(path), sdir_(dir_of(path)), r_(path) {}

  void run() {
    try {
      read_all();
    } catch (LoadError& e) {
      e.what = path_ + ":" + std::to_string(r_.line()) + ": " + e.what;
      throw;
    }
    finish();
  }

 private:
  pr_scene_file& S_;
  std::string path_, sdir_;
  Reader r_;
  Numbers num_;
  // SceneEnv::Default (scene_env.h:262-350)
  double cpos_[3] = {50.0, 52.0, 220.0}, cdir_[3] = {0.0, -0.04, -1.0}, cup_[3] = {0.0, 1.0, 0.0};
  double target_[3] = {0, 0, 0};
  std::vector<M4> camera_ms_;
  bool target_set_ = false, angle_set_ = false;
  double screen_[3] = {30.0, 30.0, 40.0}, angle_ = 0.0;
  int width_ = 320, height_ = 240, samples_ = 8, supersamples_ = 2, tent_ = 0, depth_ = 8, depth_limit_ = 64;
  int nee_ = 0, participating_ = 0, use_temp_ = 0, mlt_ = 0;
  double mutation_ = 2.0, pre_sample_ = 0.4;  // SceneEnv::Default (scene_env.h:312-313)
  float luminance_cutoff_ = 0.025f;  // a float in the reference (scene_env.h:221)
  double sensor_response_ = 1.0, doppler_ = 0.0;
  double background_[3] = {0, 0, 0}, envlight_[3] = {0, 0, 0};
  pr_medium gm_ = default_medium();
  BlackHole bh_;  // bh_.steps is the one geodesics_max_length of both blocks
  Worm wh_;
  int blackhole_disk_ = 0;  // a 'blackhole_disk' line holds for every later disk (scene_env.h:1177-1181)

  void refuse(const std::string& what) { fail("not rendered here: '" + what + "'"); }

  // a texture, map or coefficient line, read both at the top level and in a
  // BLACKHOLE block (scene_env.h:680-697, :749-763); true if it was one
  bool background_line(const std::string& b) {
    if (starts(b, "background_texture ")) {
      bh_.bg_texture = b.substr(19);
    } else if (starts(b, "map_coef ")) {
      const std::vector<double> v = num_.many(b.substr(9), 4);
      for (int i = 0; i < 4; i++) bh_.map_coef[i] = v[i];
    } else if (starts(b, "coef ")) {
      bh_.tex_coef = num_.many(b.substr(5), 1)[0];
    } else {
      return false;
    }
    return true;
  }

  void read_all() {
    std::string line;
    while (r_.get(line)) {
      const std::vector<std::string> t = tokens(line);
      if (t.empty() || line[0] == '#') continue;
      const std::string& k = t[0];
      if (t.size() == 1 && top_setting(k)) continue;
      if (starts(line, "VAR ")) {
        num_.ex.define(line.substr(4), num_.one(r_.value("VAR")));
      } else if (k == "PAHASE" && t.size() > 1) {  // the global medium keeps x, y, z
        const std::vector<double> v = num_.many(after_key(line), 3);
        for (int i = 0; i < 3; i++) gm_.phase_g[i] = v[i];
      } else if (starts(line, "BLACKHOLE")) {
        read_black_hole(line);
      } else if (starts(line, "WORMHOLE")) {
        read_wormhole();
      } else if (background_line(line)) {
      } else {
        S_.warnings += "skipped: " + line + "\n";
      }
    }
  }

  // a keyword alone on its line; false if it is not one of them
  bool top_setting(const std::string& k) {
    if (k == "IMAGE") {
      const std::string v = r_.value(k);
      std::sscanf(v.c_str(), "%d %d", &width_, &height_);
    } else if (k == "SCREEN") {
      const std::vector<double> v = num_.many(r_.value(k), 3);
      for (int i = 0; i < 3; i++) screen_[i] = v[i];
    } else if (k == "SAMPLING") {
      scan(r_.value(k), "%d", samples_);
    } else if (k == "SUPERSAMPLING") {
      scan(r_.value(k), "%d", supersamples_);
    } else if (k == "tentfilter") {
      tent_ = num_.integer(r_.value(k));
    } else if (k == "DEPTH") {
      depth_ = num_.integer(r_.value(k));
    } else if (k == "DEPTH_LIMIT") {
      depth_limit_ = num_.integer(r_.value(k));
    } else if (k == "luminance_cutoff") {
      luminance_cutoff_ = (float)num_.one(r_.value(k));
    } else if (k == "sensor_response") {
      scan(r_.value(k), "%lf", sensor_response_);
    } else if (k == "gamma_offset") {
      S_.gamma_offset = num_.one(r_.value(k));
    } else if (k == "nextEventEstimation") {
      scan(r_.value(k), "%d", nee_);
    } else if (k == "participatingMedia") {
      scan(r_.value(k), "%d", participating_);
    } else if (k == "use_accretion_disk_temperature") {
      use_temp_ = num_.integer(r_.value(k));
    } else if (k == "color_doppler_factor_effect") {
      doppler_ = num_.one(r_.value(k));
    } else if (k == "CAMERA_POS" || k == "CAMERA_DIR" || k == "CAMERA_UPVEC" || k == "TARGET_POS") {
      const std::vector<double> v = num_.many(r_.value(k), 3);
      double* d = k == "CAMERA_POS" ? cpos_ : k == "CAMERA_DIR" ? cdir_ : k == "CAMERA_UPVEC" ? cup_ : target_;
      for (int i = 0; i < 3; i++) d[i] = v[i];
      if (k == "TARGET_POS") target_set_ = true;
    } else if (k == "CAMERA_ANGLE") {
      angle_ = num_.one(r_.value(k));
      angle_set_ = true;
    } else if (k == "BACKGROUND" || k == "ENVLIGHT") {
      const std::vector<double> v = num_.many(r_.value(k), 3);
      for (int i = 0; i < 3; i++) (k == "BACKGROUND" ? background_ : envlight_)[i] = v[i];
    } else if (k == "SCATTERING" || k == "ABSORBING") {
      (void)num_.one(r_.value(k));  // the scalar: the medium set-up recomputes it from the colour
      const std::vector<double> v = num_.many(r_.value(k), 3);
      for (int i = 0; i < 3; i++) (k == "SCATTERING" ? gm_.sigma_s_rgb : gm_.sigma_a_rgb)[i] = v[i];
    } else if (k == "PAHASE") {
      const double g = num_.one(r_.value(k));
      for (int i = 0; i < 3; i++) gm_.phase_g[i] = g;
    } else if (k == "OBJECT") {
      read_object();
    } else if (k == "LENS") {
      const std::vector<double> v = num_.many(r_.value(k), 2);
      if (v[0] > 0.0) refuse("LENS " + std::to_string(v[0]));
    } else if (among(k, {"use_mollweide_projection", "special_relativity_effects"})) {
      if (num_.integer(r_.value(k)) != 0) refuse(k);
    } else if (k == "metropolisTransport") {
      scan(r_.value(k), "%d", mlt_);  // sscanf (scene_env.h:642-646)
    } else if (k == "mutation") {
      mutation_ = num_.one(r_.value(k));
    } else if (k == "pre_sample") {
      pre_sample_ = num_.one(r_.value(k));
    } else if (among(k, {"energyRedistributionPathTracing"})) {
      int on = 0;
      scan(r_.value(k), "%d", on);
      if (on != 0) refuse(k);
    } else if (k == "CAMERA_MATRIX") {  // block up to an empty line (scene_env.h:549-573)
      std::string b;
      while (r_.get(b) && !b.empty()) {
        if (starts(b, "rotation ")) {
          const std::vector<double> v = num_.many(after_key(b), 3);
          for (int a = 0; a < 3; a++) camera_ms_.push_back(rotation(a, v[a] * kRad));
        } else if (starts(b, "translate ")) {
          const std::vector<double> v = num_.many(after_key(b), 3);
          camera_ms_.push_back(translation(v[0], v[1], v[2]));
        }
      }
    } else if (among(k, {"THREAD", "IMAGEDUMP", "TIMELIMIT"})) {
      (void)num_.one(r_.value(k));  // does not change the image
    } else if (among(k, {"OUTPUT", "mlt_r1r2", "velocity"})) {
      (void)r_.value(k);  // does not change the image rendered here
    } else {
      return false;
    }
    return true;
  }

  void read_black_hole(const std::string& line) {
    bh_.exists = true;
    if (starts(line, "BLACKHOLE ")) {
      const std::vector<double> v = num_.many(after_key(line), 3);
      for (int i = 0; i < 3; i++) bh_.pos[i] = v[i];
      bh_.pos_set = true;
    }
    std::string b;
    while (r_.raw(b) && !b.empty()) {
      if (b[0] == '#') continue;
      if (background_line(b)) continue;
      if (starts(b, "dist ")) {
        bh_.dist = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "geodesics_max_length ")) {
        bh_.steps = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "accretion_disk ")) {
        bh_.rdisk = num_.many(after_key(b), 1)[0];  // the disk lookup takes the disk entity's radius
      } else if (starts(b, "angular_momentum ")) {
        bh_.a = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "initial_condition ")) {
        bh_.init_cond = (int)num_.many(after_key(b), 1)[0];
      } else if (starts(b, "accretion_disk_texture ")) {
        if (bh_.disk_texture.empty())
          bh_.disk_texture = b.substr(23);
        else
          S_.warnings += "only the first accretion_disk_texture is read: " + b + "\n";
      } else if (!tokens(b).empty()) {
        S_.warnings += "skipped in BLACKHOLE: " + b + "\n";
      }
    }
  }

  void read_wormhole() {
    wh_.exists = true;
    std::string b;
    while (r_.raw(b) && !b.empty()) {
      if (b[0] == '#') continue;
      if (starts(b, "in ") || starts(b, "out ")) {
        const std::vector<double> v = num_.many(after_key(b), 3);
        for (int i = 0; i < 3; i++) (starts(b, "in ") ? wh_.in : wh_.out)[i] = v[i];
        wh_.pos_set = true;
      } else if (starts(b, "Rho ")) {
        wh_.rho = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "a ")) {
        wh_.a = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "W ")) {
        wh_.w = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "sign ")) {
        wh_.sign = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "dist ")) {
        wh_.dist = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "geodesics_max_length ")) {
        bh_.steps = num_.many(after_key(b), 1)[0];
      } else if (starts(b, "background_texture1 ") || starts(b, "background_texture2 ")) {
        wh_.texture[b[18] == '1' ? 0 : 1] = b.substr(20);
      } else if (starts(b, "map_coef1 ") || starts(b, "map_coef2 ")) {
        const std::vector<double> v = num_.many(b.substr(10), 4);
        for (int i = 0; i < 4; i++) wh_.map_coef[b[8] == '1' ? 0 : 1][i] = v[i];
      } else if (starts(b, "coef1 ") || starts(b, "coef2 ")) {
        wh_.coef[b[4] == '1' ? 0 : 1] = num_.many(b.substr(6), 1)[0];
      } else if (!tokens(b).empty()) {
        S_.warnings += "skipped in WORMHOLE: " + b + "\n";
      }
    }
  }

  void read_object() {
    std::string g;
    if (!r_.get(g)) fail("OBJECT without a shape line");
    pr_entity e;
    memset(&e, 0, sizeof(e));
    e.normal_inverse = 1;
    e.mesh = -1;
    e.normal[2] = 1.0;
    e.spot_attenuation[2] = 1.0;  // the parser's defaults (scene_env.h:877-884)
    ObjMesh mesh;
    if (starts(g, "infinity_light ")) {  // a direction, used as given (scene_env.h:891-894)
      const std::vector<double> v = num_.many(after_key(g), 3);
      e.type = PR_ENT_INF_LIGHT;
      for (int i = 0; i < 3; i++) e.light_dir[i] = v[i];
    } else if (starts(g, "sphere ") || starts(g, "hemisphere ")) {
      const std::vector<double> v = num_.many(after_key(g), 4);
      e.type = PR_ENT_SPHERE;
      e.hemisphere = starts(g, "hemisphere ") ? 1 : 0;  // scene_env.h:935-939
      for (int i = 0; i < 3; i++) e.p[i] = v[i];
      e.radius = v[3];
    } else if (starts(g, "uvplane ")) {
      const std::vector<double> v = num_.many(after_key(g), 3);
      e.type = PR_ENT_UVPLANE;
      for (int i = 0; i < 3; i++) e.p[i] = v[i];
      for (int q = 0; q < 2; q++) {
        std::string uv;
        if (!r_.get(uv)) fail("uvplane needs U and V lines");
        const std::vector<double> w = num_.many(after_key(uv), 3);
        double* dst = (!uv.empty() && uv[0] == 'U') ? e.u : e.v;
        for (int i = 0; i < 3; i++) dst[i] = w[i];
      }
    } else if (starts(g, "disk ") || starts(g, "disk2 ")) {
      const bool two = g[4] == '2';
      const std::vector<double> v = num_.many(after_key(g), two ? 5 : 4);
      e.type = PR_ENT_CIRCLE;
      for (int i = 0; i < 3; i++) e.p[i] = v[i];
      e.radius = v[3];
      e.radius_inner = two ? v[4] : 0.0;
      std::string nl;
      if (!r_.get(nl)) fail("disk needs a normal line");
      const std::vector<double> n = num_.many(after_key(nl), 3);
      for (int i = 0; i < 3; i++) e.normal[i] = n[i];
    } else if (starts(g, "objfile ")) {
      e.type = PR_ENT_POLYGON;
      read_obj(resolve(g.substr(8), sdir_), mesh);
    } else {
      fail("shape not rendered here: '" + g + "'");
    }
    pr_material m = default_material();
    double material_scale = 1.0, scattering = 0.0;
    std::vector<M4> ms;
    ObjTex tx;
    std::string b;
    while (r_.raw(b) && !b.empty()) {
      if (b[0] == '#') continue;
      const std::vector<std::string> bt = tokens(b);
      if (bt.empty()) continue;
      if (bt.size() == 1 && object_setting(bt[0], m, material_scale, scattering)) continue;
      if (texture_line(b, bt, m, tx)) continue;
      object_line(b, bt, e, m, ms);
    }
    if (is_sss(m.type) && !(scattering > kEps))
      fail("a subsurface material needs a SCATTERING value above 1e-6 (the reference leaves its medium unset)");
    m.medium.scale = material_scale;
    if (e.type == PR_ENT_CIRCLE) e.blackhole_disk = blackhole_disk_;
    if (!ms.empty()) {
      if (e.type == PR_ENT_SPHERE) {  // Sphere::MatrixTransformation: the centre only
        for (const M4& mm : ms) {
          double o[3];
          apply(mm, e.p, o);
          for (int i = 0; i < 3; i++) e.p[i] = o[i];
        }
      } else if (e.type != PR_ENT_POLYGON) {
        fail("rotation / translate / scale of a uvplane or disk is not rendered here");
      }
    }
    if (e.type == PR_ENT_POLYGON) {
      // Obj's normals are made at load (ObjLoader.cpp:493), then moved with
      // the vertices (Polygon::MatrixTransformation)
      std::vector<float> fn, vn;
      std::vector<int32_t> fvn;
      const int nf = (int)(mesh.f.size() / 3);
      if (!mesh.vn.empty()) {
        face_normals_from_vn(mesh, fn);
        vn = mesh.vn;
        fvn = mesh.nid;
      } else if (!ms.empty()) {
        pr::face_normals(mesh.v.data(), mesh.f.data(), nf, fn);
        if (e.smooth) {
          pr::vertex_normals(mesh.v.data(), mesh.f.data(), nf, (int)(mesh.v.size() / 3), vn);
          fvn = mesh.f;
        }
      }
      transform_mesh(ms, mesh.v, fn, vn);
      if (tx.tex_alpha) fail("a 32-bit texture with transparent texels on a mesh (the reference's alpha test) is not rendered here");
      e.mesh = (int)S_.verts.size();
      S_.verts.push_back(std::move(mesh.v));
      S_.faces.push_back(std::move(mesh.f));
      S_.fnormals.push_back(std::move(fn));
      S_.vnormals.push_back(std::move(vn));
      S_.face_vn.push_back(std::move(fvn));
      S_.uvs.push_back(std::move(mesh.vt));
      S_.face_uv.push_back(std::move(mesh.tid));
      S_.omats.push_back(std::move(mesh.mats));
      S_.omat_tex.push_back(std::move(mesh.mat_tex));
      S_.fmat.push_back(std::move(mesh.fmat));
    }
    e.material = (int)S_.mats.size();
    S_.mats.push_back(m);
    S_.tex8.push_back(std::move(tx.tex8));
    S_.ibl8.push_back(std::move(tx.ibl8));
    S_.iblf.push_back(std::move(tx.iblf));
    S_.bump8.push_back(std::move(tx.bump8));
    S_.ents.push_back(e);
  }

  // an OBJECT's images (scene_env.h:984-1175): texture, ibl_texture (BMP or
  // Radiance HDR), ibl_texture_coef, repeat and the four sphere mappings
  struct ObjTex {
    std::vector<uint8_t> tex8, ibl8, bump8;
    std::vector<float> iblf;
    bool tex_alpha = false;  // the texture has texels with alpha below 255 (read by mesh hits)
  };
  bool texture_line(const std::string& b, const std::vector<std::string>& bt, pr_material& m, ObjTex& tx) {
    const std::string& k = bt[0];
    if (k == "texture" && bt.size() >= 2) {
      int w = 0, h = 0;
      std::vector<uint8_t> rgba;
      read_bmp(resolve(b.substr(8), sdir_), 4, rgba, w, h);
      tx.tex8.resize(3 * (size_t)w * h);
      tx.tex_alpha = false;
      for (size_t q = 0; q < (size_t)w * h; q++) {
        for (int a = 0; a < 3; a++) tx.tex8[3 * q + a] = rgba[4 * q + a];
        tx.tex_alpha |= rgba[4 * q + 3] != 255;
      }
      m.texture_width = w;
      m.texture_height = h;
    } else if (k == "ibl_texture" && bt.size() >= 2) {
      const std::string file = resolve(b.substr(12), sdir_);
      std::string ext = file.size() >= 4 ? file.substr(file.size() - 4) : std::string();
      for (char& ch : ext) ch = (char)std::tolower((unsigned char)ch);
      int w = 0, h = 0;
      if (ext == ".bmp") {
        read_bmp(file, 3, tx.ibl8, w, h);
        tx.iblf.clear();
      } else if (ext == ".hdr") {
        read_hdr(file, tx.iblf, w, h);
        tx.ibl8.clear();
      } else {
        fail("ibl_texture takes a .bmp or .hdr file: " + file);
      }
      m.ibl_width = w;
      m.ibl_height = h;
    } else if (k == "bump_texture" && bt.size() >= 2) {
      int w = 0, h = 0;
      read_bmp(resolve(b.substr(13), sdir_), 3, tx.bump8, w, h);
      m.bump_width = w;
      m.bump_height = h;
    } else if (k == "ibl_texture_coef") {
      m.ibl_coef = num_.many(after_key(b), 1)[0];
    } else if (k == "repeat") {
      scan(b, "repeat %d", m.repeat);
    } else if (k == "hemisphere_map" || k == "angular_map" || k == "panoramic_map" || k == "equirectangular_map") {
      int on = 0;
      scan(after_key(b), "%d", on);
      const int bit = k == "hemisphere_map" ? PR_MAP_HEMISPHERE
                      : k == "angular_map"  ? PR_MAP_ANGULAR
                      : k == "panoramic_map" ? PR_MAP_PANORAMIC
                                             : PR_MAP_EQUIRECTANGULAR;
      // the flag is a char set from the value (scene_env.h:1135-1162)
      m.map_flags = ((char)on != 0) ? (m.map_flags | bit) : (m.map_flags & ~bit);
    } else {
      return false;
    }
    return true;
  }

  // an OBJECT keyword alone on its line, value on the next (scene_env.h:1257-1367)
  bool object_setting(const std::string& k, pr_material& m, double& material_scale, double& scattering) {
    if (k == "SCATTERING" || k == "ABSORBING") {
      const double s = num_.one(r_.value(k));
      if (k == "SCATTERING") scattering = s;
      const std::vector<double> v = num_.many(r_.value(k), 3);
      for (int i = 0; i < 3; i++) (k == "SCATTERING" ? m.medium.sigma_s_rgb : m.medium.sigma_a_rgb)[i] = v[i];
    } else if (k == "PAHASE") {
      const double g = num_.one(r_.value(k));
      for (int i = 0; i < 3; i++) m.medium.phase_g[i] = g;
    } else if (k == "level") {
      m.medium.level = num_.integer(r_.value(k));
      if (m.medium.level == -2) m.medium.use_bssrdf = 1;
      if (m.medium.level >= 0) m.medium.use_bssrdf = 0;
    } else if (k == "BSSRDF") {
      m.medium.use_bssrdf = num_.integer(r_.value(k));
      std::string skip;
      (void)r_.get(skip);
    } else if (k == "MATERIAL_R_MAX") {
      m.medium.r_max = num_.one(r_.value(k));
    } else if (k == "MATERIAL_SCALE") {
      material_scale = num_.one(r_.value(k));
    } else if (k == "MATERIAL_SYMBOL") {
      refuse("MATERIAL_SYMBOL " + r_.value(k));
    } else {
      return false;
    }
    return true;
  }

  // The reference reads an OBJECT block's 'PAHASE x y z' and 'rotation x y
  // z' values into the same three variables that hold a sphere's or disk's
  // centre, and builds the shape from them after the block
  // (scene_env.h:1349-1375, :1621, :1672): such a line moves the centre to
  // its own three values, before any transform.
  static void shared_xyz(pr_entity& e, const std::vector<double>& v) {
    if (e.type == PR_ENT_SPHERE || e.type == PR_ENT_CIRCLE)
      for (int i = 0; i < 3; i++) e.p[i] = v[i];
  }

  // an OBJECT line with its values on the same line (scene_env.h:977-1520)
  void object_line(const std::string& b, const std::vector<std::string>& bt, pr_entity& e, pr_material& m,
                   std::vector<M4>& ms) {
    const std::string& k = bt[0];
    if (k == "emission" || k == "color" || k == "specular") {
      const std::vector<double> v = num_.many(after_key(b), 3);
      double* dst = k == "emission" ? m.emission : k == "color" ? m.color : m.specular;
      for (int i = 0; i < 3; i++) dst[i] = v[i];
    } else if (k == "roughness") {
      m.roughness = num_.many(after_key(b), 1)[0];
    } else if (k == "refractive_index") {
      m.refractive_index = num_.many(after_key(b), 1)[0];
    } else if (k == "r_refractive_index") {
      m.r_refractive_index = num_.many(after_key(b), 1)[0];
    } else if (k == "ward_brdf") {  // colour and specular scaled by lo_d, lo_s (scene_env.h:1417-1425)
      const std::vector<double> v = num_.many(after_key(b), 4);
      for (int i = 0; i < 3; i++) {
        m.color[i] = m.color[i] * v[0];
        m.specular[i] = m.specular[i] * v[1];
      }
      m.ward_alpha[0] = v[2];
      m.ward_alpha[1] = v[3];
    } else if (k == "phong_brdf") {  // scene_env.h:1427-1435
      const std::vector<double> v = num_.many(after_key(b), 3);
      for (int i = 0; i < 3; i++) {
        m.color[i] = m.color[i] * v[0];
        m.specular[i] = m.specular[i] * v[1];
      }
      m.phong_exponent = v[2];
    } else if (k == "reflection" && bt.size() == 2) {  // scene_env.h:1444-1520
      const std::string& rt = bt[1];
      if (rt == "diffuse") {
        m.type = PR_MAT_DIFFUSE;
        m.roughness = 1.0;
      } else if (rt == "specular") {
        m.type = PR_MAT_SPECULAR;
        m.roughness = 0.0;
      } else if (rt == "reflection") {
        m.type = PR_MAT_REFRACTION;
        if (m.refractive_index == 0.0) {
          m.refractive_index = 1.5;
          m.r_refractive_index = 1.5 / 1.000292;
        }
      } else if (rt == "ward_brdf") {
        m.type = PR_MAT_WARD;
      } else if (rt == "phong_brdf") {
        m.type = PR_MAT_PHONG;
      } else if (rt == "Subsurface_Scattering") {
        m.type = m.type == PR_MAT_REFRACTION ? PR_MAT_SSS_REFRACTION
                 : m.type == PR_MAT_WARD    ? PR_MAT_SSS_WARD
                                            : PR_MAT_SSS_DIFFUSE;
      } else {
        refuse(b);  // dispersion formulas
      }
    } else if (k == "PAHASE") {  // in an OBJECT block the reference keeps x for y (scene_env.h:1349-1355)
      const std::vector<double> v = num_.many(after_key(b), 3);
      m.medium.phase_g[0] = v[0];
      m.medium.phase_g[1] = v[0];
      m.medium.phase_g[2] = v[2];
      shared_xyz(e, v);
    } else if (k == "rotation") {
      const std::vector<double> v = num_.many(after_key(b), 3);
      for (int a = 0; a < 3; a++) ms.push_back(rotation(a, v[a] * kRad));
      shared_xyz(e, v);
    } else if (k == "translate") {
      const std::vector<double> v = num_.many(after_key(b), 3);
      ms.push_back(translation(v[0], v[1], v[2]));
    } else if (k == "scale") {
      const std::vector<double> v = num_.many(after_key(b), 3);
      ms.push_back(scaling(v[0], v[1], v[2]));
    } else if (k == "normal") {
      scan(b, "normal %d", e.normal_inverse);
    } else if (k == "disk_map") {
      scan(b, "disk_map %d", m.disk_map);
    } else if (k == "blackhole_disk") {
      scan(b, "blackhole_disk %d", blackhole_disk_);
    } else if (k == "parallel_light") {
      scan(b, "parallel_light %d", e.parallel_light);
    } else if (k == "spot_light") {
      scan(b, "spot_light %d", e.spot_light);
    } else if (k == "parallel_light_dir" || k == "spot_light_dir") {
      // one direction for both keywords, normalised as read (scene_env.h:1216-1234)
      const std::vector<double> v = num_.many(after_key(b), 3);
      const double inv = 1.0 / std::sqrt((v[0] * v[0] + v[2] * v[2]) + v[1] * v[1]);
      for (int i = 0; i < 3; i++) e.light_dir[i] = v[i] * inv;
    } else if (k == "spot_light_angle") {
      const std::vector<double> v = num_.many(after_key(b), 2);
      e.spot_angle[0] = v[0];
      e.spot_angle[1] = v[1];
    } else if (k == "spot_light_falloff") {
      e.spot_falloff = num_.many(after_key(b), 1)[0];
    } else if (k == "spot_attenuation") {
      const std::vector<double> v = num_.many(after_key(b), 3);
      for (int i = 0; i < 3; i++) e.spot_attenuation[i] = v[i];
    } else if (k == "smooth") {
      scan(after_key(b), "%d", e.smooth);  // sscanf "smooth %d" (scene_env.h:1195-1198)
    } else if (among(k, {"background", "shadow"})) {
      int on = 0;
      scan(after_key(b), "%d", on);
      if (on != 0) refuse(b);
    } else if (k == "media_ignore_front_back") {
      if ((int)num_.many(after_key(b), 1)[0] != 0) refuse(b);
    } else if (among(k, {"texture", "bump_texture", "ibl_texture"})) {
      refuse(b);  // an image keyword without a file
    } else if (among(k, {"back"})) {
      // not read by anything rendered here
    } else {
      S_.warnings += "skipped in OBJECT: " + b + "\n";
    }
  }

  // end of SceneEnv::Load (scene_env.h:1862-1921, :2056-2098)
  void finish() {
    double dir[3] = {cdir_[0], cdir_[1], cdir_[2]};
    auto normalise = [](double* v) {
      const double inv = 1.0 / std::sqrt((v[0] * v[0] + v[2] * v[2]) + v[1] * v[1]);
      for (int i = 0; i < 3; i++) v[i] = v[i] * inv;
    };
    if (target_set_) {  // the direction towards TARGET_POS, normalised (and once more below)
      for (int i = 0; i < 3; i++) dir[i] = target_[i] - cpos_[i];
      normalise(dir);
    }
    if (!camera_ms_.empty()) {
      // CAMERA_MATRIX: each matrix moves a tracked origin, the direction
      // taken relative to it, and the position (the up vector stays)
      double org[3] = {0, 0, 0}, o[3];
      for (const M4& m : camera_ms_) {
        apply(m, org, o);
        for (int i = 0; i < 3; i++) org[i] = o[i];
        const double rel[3] = {dir[0] - org[0], dir[1] - org[1], dir[2] - org[2]};
        apply(m, rel, dir);
        apply(m, cpos_, o);
        for (int i = 0; i < 3; i++) cpos_[i] = o[i];
      }
      normalise(dir);
    }
    normalise(dir);
    pr_camera& cam = S_.cam;
    memset(&cam, 0, sizeof(cam));
    for (int i = 0; i < 3; i++) {
      cam.position[i] = cpos_[i];
      cam.dir[i] = dir[i];
      cam.up[i] = cup_[i];
    }
    cam.screen_width = screen_[0];
    cam.screen_height = screen_[1];
    cam.screen_dist = screen_[2];
    if (angle_set_) {
      cam.screen_width = 2.0 * screen_[2] * std::tan(angle_ * kRad / 2.0);
      cam.screen_height = cam.screen_width;
    }
    cam.width = width_;
    cam.height = height_;
    if (width_ <= 0 || height_ <= 0) fail("IMAGE must give a positive width and height");

    pr_render_params& p = S_.prm;
    memset(&p, 0, sizeof(p));
    p.samples = samples_;
    p.supersamples = supersamples_;
    p.tent_filter = tent_;
    p.depth = depth_;
    p.depth_limit = depth_limit_;
    p.nee = nee_;
    p.mode = PR_MODE_MEGAKERNEL;
    if (mlt_) {
      // the MLT set-up (scene_env.h:1946-1957): default seeds and mutations
      // for non-positive values, the tent filter; its 1/4 sensor scale is
      // part of the PR_MODE_MLT estimator
      p.mode = PR_MODE_MLT;
      p.tent_filter = 1;
      if (pre_sample_ <= 0.0) pre_sample_ = 0.4;
      if (mutation_ <= 0.0) mutation_ = 32;
    }
    p.mlt_mutation = mutation_;
    p.mlt_pre_sample = pre_sample_;
    p.luminance_cutoff = (double)luminance_cutoff_;
    p.sensor_response = sensor_response_;
    // participatingMedia is cleared when the global medium has no extinction
    // (ParticipatingMediaPrm.h:139-145)
    const double sig_t = (gm_.sigma_s_rgb[0] + gm_.sigma_s_rgb[1] + gm_.sigma_s_rgb[2]) / 3 +
                         (gm_.sigma_a_rgb[0] + gm_.sigma_a_rgb[1] + gm_.sigma_a_rgb[2]) / 3;
    if (sig_t < 1.0e-12) participating_ = 0;
    p.media = participating_;

    S_.meshes.resize(S_.verts.size());
    for (size_t i = 0; i < S_.verts.size(); i++) {
      pr_mesh& mm = S_.meshes[i];
      memset(&mm, 0, sizeof(mm));
      mm.n_vertices = (int32_t)(S_.verts[i].size() / 3);
      mm.n_faces = (int32_t)(S_.faces[i].size() / 3);
      mm.vertices = S_.verts[i].data();
      mm.faces = S_.faces[i].data();
      mm.face_normals = S_.fnormals[i].empty() ? nullptr : S_.fnormals[i].data();
      if (!S_.vnormals[i].empty()) {
        mm.n_vertex_normals = (int32_t)(S_.vnormals[i].size() / 3);
        mm.vertex_normals = S_.vnormals[i].data();
        mm.face_vn = S_.face_vn[i].data();
      }
      if (!S_.uvs[i].empty() && !S_.face_uv[i].empty()) {
        mm.n_uv = (int32_t)(S_.uvs[i].size() / 2);
        mm.uv = S_.uvs[i].data();
        mm.face_uv = S_.face_uv[i].data();
      }
      if (!S_.omats[i].empty() && !S_.fmat[i].empty()) {
        for (size_t k = 0; k < S_.omats[i].size(); k++)
          S_.omats[i][k].texture = S_.omat_tex[i][k].empty() ? nullptr : S_.omat_tex[i][k].data();
        mm.n_obj_materials = (int32_t)S_.omats[i].size();
        mm.obj_materials = S_.omats[i].data();
        mm.face_obj_material = S_.fmat[i].data();
      }
    }
    pr_scene_desc& d = S_.desc;
    memset(&d, 0, sizeof(d));
    d.n_materials = (int32_t)S_.mats.size();
    d.n_entities = (int32_t)S_.ents.size();
    d.n_meshes = (int32_t)S_.meshes.size();
    d.participating_media = participating_;
    for (size_t i = 0; i < S_.mats.size(); i++) {
      pr_material& mm = S_.mats[i];
      mm.texture = S_.tex8[i].empty() ? nullptr : S_.tex8[i].data();
      mm.ibl_rgb8 = S_.ibl8[i].empty() ? nullptr : S_.ibl8[i].data();
      mm.ibl_rgbf = S_.iblf[i].empty() ? nullptr : S_.iblf[i].data();
      mm.bump = S_.bump8[i].empty() ? nullptr : S_.bump8[i].data();
    }
    d.materials = S_.mats.data();
    d.entities = S_.ents.data();
    d.meshes = S_.meshes.data();
    for (int i = 0; i < 3; i++) {
      d.background[i] = background_[i];
      d.environment_light[i] = envlight_[i];
    }
    d.medium = gm_;
    pr_wormhole& ww = d.wormhole;
    memset(&ww, 0, sizeof(ww));
    ww.texture_coef[0] = ww.texture_coef[1] = 1.0;
    if (wh_.exists) {
      // without a mouth position 'in' sits dist along the camera direction
      // (scene_env.h:2100-2110); the frame is built from CAMERA_POS
      if (!wh_.pos_set)
        for (int i = 0; i < 3; i++) wh_.in[i] = cpos_[i] + dir[i] * wh_.dist;
      ww.enabled = 1;
      ww.max_steps = (int32_t)bh_.steps;
      for (int i = 0; i < 3; i++) {
        ww.in[i] = wh_.in[i];
        ww.out[i] = wh_.out[i];
        ww.camera[i] = cpos_[i];
      }
      ww.rho = wh_.rho;
      ww.a = wh_.a;
      ww.w = wh_.w;
      ww.sign = (int32_t)wh_.sign;
      for (int k = 0; k < 2; k++) {
        for (int i = 0; i < 4; i++) ww.map_coef[k][i] = wh_.map_coef[k][i];
        ww.texture_coef[k] = wh_.coef[k];
        if (wh_.texture[k].empty()) continue;
        int w = 0, h = 0;
        read_bmp(resolve(wh_.texture[k], sdir_), 3, S_.worm_tex[k], w, h);
        ww.texture[k] = S_.worm_tex[k].data();
        ww.texture_width[k] = w;
        ww.texture_height[k] = h;
      }
    }
    pr_kerr& kk = d.kerr;
    memset(&kk, 0, sizeof(kk));
    kk.texture_coef = 1.0;
    if (!bh_.exists) return;
    if (bh_.init_cond != 0) fail("BLACKHOLE initial_condition other than 0 is not rendered here");
    // without a position the black hole sits dist along the camera direction
    if (!bh_.pos_set)
      for (int i = 0; i < 3; i++) bh_.pos[i] = cpos_[i] + dir[i] * bh_.dist;
    kk.enabled = 1;
    kk.max_steps = (int32_t)bh_.steps;
    for (int i = 0; i < 3; i++) {
      kk.position[i] = bh_.pos[i];
      kk.observer[i] = cpos_[i];
    }
    kk.a = bh_.a;
    for (int i = 0; i < 4; i++) kk.map_coef[i] = bh_.map_coef[i];
    kk.texture_coef = bh_.tex_coef;
    kk.precision = PR_KERR_FP64;
    kk.use_accretion_disk_temperature = use_temp_;
    kk.color_doppler_factor_effect = doppler_;
    kk.disk_seed = 1;  // the reference seeds its scene generator from the clock
    if (!bh_.bg_texture.empty()) {
      int w = 0, h = 0;
      read_bmp(resolve(bh_.bg_texture, sdir_), 3, S_.bg_tex, w, h);
      kk.texture = S_.bg_tex.data();
      kk.texture_width = w;
      kk.texture_height = h;
    }
    if (!bh_.disk_texture.empty()) {
      int w = 0, h = 0;
      read_bmp(resolve(bh_.disk_texture, sdir_), 4, S_.disk_tex, w, h);
      kk.disk_texture = S_.disk_tex.data();
      kk.disk_texture_width = w;
      kk.disk_texture_height = h;
    }
  }
};

}  // namespace

extern "C" {

pr_scene_file* pr_scene_file_load(const char* path, char* err, int errlen) {
  if (err && errlen > 0) err[0] = '\0';
  auto* S = new pr_scene_file();
  try {
    if (!path) fail("null path");
    Loader(*S, path).run();
  } catch (const LoadError& e) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.what.c_str());
    delete S;
    return nullptr;
  } catch (const std::exception& e) {
    if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.what());
    delete S;
    return nullptr;
  }
  return S;
}

const pr_scene_desc* pr_scene_file_desc(const pr_scene_file* f) { return f ? &f->desc : nullptr; }

int pr_scene_file_camera(const pr_scene_file* f, pr_camera* cam, pr_render_params* prm, double* gamma_offset) {
  if (!f) return PR_E_ARG;
  if (cam) *cam = f->cam;
  if (prm) *prm = f->prm;
  if (gamma_offset) *gamma_offset = f->gamma_offset;
  return PR_OK;
}

const char* pr_scene_file_warnings(const pr_scene_file* f) { return f ? f->warnings.c_str() : ""; }

void pr_scene_file_free(pr_scene_file* f) { delete f; }

}  // extern "C"
