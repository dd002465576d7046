// Command-line harness around the reference renderer (Sanaxen/prender).
//
// Test infrastructure only: oracle/build_ref.sh compiles this file together
// with the reference's own translation units into oracle/_ref/prender_ref.
// It runs the reference code unchanged and writes its results as raw binary
// so that the Python tests can freeze golden fixtures from them.
//
//   prender_ref render   <scene.txt> <image.f64>          Render::Run() (render.h:1125), or
//                                                          Render::RunMLT() (render.h:363) for a
//                                                          scene with metropolisTransport 1
//   prender_ref firsthit <scene.txt> <rays.f64> <out.bin>  intersect_scene_ (scene.cpp:83)
//                                                          + QBVH::CheckIntersection (QBVH.cpp:17)
//   prender_ref qbvh     <scene.txt> <entity> <out.bin>    QBVH node + leaf arrays (QBVH.h:53)
//   prender_ref kerr     <scene.txt> <rays.f64> <out.bin>  intersect_scene Kerr branch (scene.cpp:448),
//                                                          with the hit point's colour and emission
//   prender_ref radiance <scene.txt> <rays.f64> <out.f64> <seed>
//                                                          radiance() roots (radiance.h:25)
//   prender_ref hdr      <scene.txt> <image.f64> <out.hdr>  Render::OutputHdr (render.h:1649) of a given
//                                                          image (the scene's size, W*H*3 doubles)
//
// The reference keeps members private; the harness opens them up for reading.
#include <omp.h>
#define private public
#define protected public
#include "scene.h"
#include "render.h"
#include "scene_env.h"
#undef private
#undef protected
#include <cstdint>
#include <vector>

using namespace prender;

void init_prime_numbers();  // QMC.cpp:7

thread_local KerrProbe prender_kerr_probe;

static std::vector<double> read_f64(const char* path) {
  std::vector<double> v;
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(3); }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  v.resize(n / sizeof(double));
  if (fread(v.data(), sizeof(double), v.size(), f) != v.size()) exit(3);
  fclose(f);
  return v;
}

static FILE* wopen(const char* path) {
  FILE* f = fopen(path, "wb");
  if (!f) { fprintf(stderr, "cannot write %s\n", path); exit(3); }
  return f;
}

// The scene's own generator (SceneEnv::rand_, scene_env.h:213), which the
// entities' alpha tests draw from (the accretion disk, circle.h:331), is
// seeded from the clock (scene_env.h:306); PRENDER_SCENE_RAND_SEED reseeds it
// through its public seed() so that one-thread runs are reproducible.
static SceneEnv* load(const char* scene) {
  SceneEnv* env = new SceneEnv();
  env->Load(const_cast<char*>(scene));
  CreateEntList(*env);
  if (const char* sd = getenv("PRENDER_SCENE_RAND_SEED")) env->rand_.seed((unsigned)strtoul(sd, nullptr, 10));
  return env;
}

int main(int argc, char** argv) {
  if (argc < 3) { fprintf(stderr, "usage: prender_ref <cmd> <scene> ...\n"); return 2; }
  std::string cmd = argv[1];
  if (cmd == "render" && argc >= 4) {
    SceneEnv* env = load(argv[2]);
    Render r(*env);
    // main.cpp:48, :193-196: RunMLT seeds its primary-sample generators
    // from the prime table (built before the timed region)
    if (env->metropolisTransport) ::init_prime_numbers();
    double t0 = omp_get_wtime();
    if (env->metropolisTransport) {
      r.RunMLT();
    } else {
      r.Run();
    }
    double t1 = omp_get_wtime();
    int w = env->image_width, h = env->image_height;
    // Render's first two data members (render.h:163-164) are implicitly
    // private; read the accumulated image through a layout-identical view.
    struct RenderView { SceneEnv* env_p; Color* image; };
    const Color* image = reinterpret_cast<RenderView*>(&r)->image;
    FILE* f = wopen(argv[3]);
    for (int i = 0; i < w * h; i++) {
      double c[3] = {image[i].x, image[i].y, image[i].z};
      fwrite(c, sizeof(double), 3, f);
    }
    fclose(f);
    printf("{\"run_seconds\": %.6f, \"threads\": %d, \"width\": %d, \"height\": %d}\n",
           t1 - t0, env->threads, w, h);
    return 0;
  }
  if (cmd == "firsthit" && argc >= 5) {
    SceneEnv* env = load(argv[2]);
    std::vector<double> rays = read_f64(argv[3]);
    size_t n = rays.size() / 6;
    FILE* f = wopen(argv[4]);
    for (size_t k = 0; k < n; k++) {
      Ray ray(Vector3d(rays[6 * k], rays[6 * k + 1], rays[6 * k + 2]),
              Vector3d(rays[6 * k + 3], rays[6 * k + 4], rays[6 * k + 5]));
      Intersection isect;
      bool hit = intersect_scene_(ray, &isect, 0);
      int32_t ent = hit ? isect.object_id : -1;
      int32_t prim = -1;
      if (hit && EntList->List[ent]->qbvh) {
        // same offset origin as intersect_scene_ (scene.cpp:92)
        const Ray ray2(ray.org + ray.dir * 0.000001, ray.dir);
        Intersection h2;
        if (EntList->List[ent]->qbvh->CheckIntersection(ray2, h2)) prim = h2.object_id;
      }
      double t = hit ? isect.hitpoint.distance : -1.0;
      fwrite(&ent, 4, 1, f);
      fwrite(&prim, 4, 1, f);
      fwrite(&t, 8, 1, f);
      double pn[6] = {isect.hitpoint.position.x, isect.hitpoint.position.y, isect.hitpoint.position.z,
                      isect.hitpoint.normal.x,   isect.hitpoint.normal.y,   isect.hitpoint.normal.z};
      fwrite(pn, 8, 6, f);
    }
    fclose(f);
    return 0;
  }
  if (cmd == "qbvh" && argc >= 5) {
    SceneEnv* env = load(argv[2]);
    int e = atoi(argv[3]);
    QBVH* q = EntList->List[e]->qbvh;
    if (!q) { fprintf(stderr, "entity %d has no QBVH\n", e); return 4; }
    FILE* f = wopen(argv[4]);
    int64_t nn = (int64_t)q->m_usedNodeCount, nl = (int64_t)q->m_leafObjectArray.size();
    fwrite(&nn, 8, 1, f);
    fwrite(&nl, 8, 1, f);
    for (int64_t i = 0; i < nn; i++) {
      const QBVH::QBVH_structure& nd = q->m_root.get()[i];
      float b[2][3][4];
      for (int m = 0; m < 2; m++)
        for (int a = 0; a < 3; a++) _mm_storeu_ps(b[m][a], nd.bboxes[m][a]);
      fwrite(b, 4, 24, f);
      for (int c = 0; c < 4; c++) { uint64_t ch = (uint64_t)nd.children[c]; fwrite(&ch, 8, 1, f); }
      int32_t ax[3] = {nd.axis_top, nd.axis_left, nd.axis_right};
      fwrite(ax, 4, 3, f);
    }
    for (int64_t i = 0; i < nl; i++) {
      int32_t id = q->m_leafObjectArray[i] ? q->m_leafObjectArray[i]->id : -1;
      fwrite(&id, 4, 1, f);
    }
    fclose(f);
    return 0;
  }
  if (cmd == "kerr" && argc >= 5) {
    SceneEnv* env = load(argv[2]);
    std::vector<double> rays = read_f64(argv[3]);
    size_t n = rays.size() / 6;
    FILE* f = wopen(argv[4]);
    for (size_t k = 0; k < n; k++) {
      Ray ray(Vector3d(rays[6 * k], rays[6 * k + 1], rays[6 * k + 2]),
              Vector3d(rays[6 * k + 3], rays[6 * k + 4], rays[6 * k + 5]));
      prender_kerr_probe = KerrProbe();
      Intersection isect;
      bool hit = intersect_scene(ray, &isect, 0);
      int32_t obj = isect.object_id;
      int32_t h = hit ? 1 : 0;
      fwrite(&obj, 4, 1, f);
      fwrite(&h, 4, 1, f);
      const KerrProbe& p = prender_kerr_probe;
      double rec[16] = {(double)p.reached_end, (double)p.steps,
                        p.y[0], p.y[1], p.y[2], p.y[3], p.y[4], p.y[5],
                        p.org[0], p.org[1], p.org[2], p.dir[0], p.dir[1], p.dir[2],
                        hit ? isect.hitpoint.distance : -1.0, 0.0};
      fwrite(rec, 8, 16, f);
      double col[6] = {isect.hitpoint.material.color.x,    isect.hitpoint.material.color.y,
                       isect.hitpoint.material.color.z,    isect.hitpoint.material.emission.x,
                       isect.hitpoint.material.emission.y, isect.hitpoint.material.emission.z};
      fwrite(col, 8, 6, f);
    }
    fclose(f);
    return 0;
  }
  if (cmd == "radiance" && argc >= 6) {
    // One radiance() root per input ray, all from one MT19937-64 stream seeded
    // with <seed> (the per-thread streams of Render::Run are seeded i+1).
    SceneEnv* env = load(argv[2]);
    std::vector<double> rays = read_f64(argv[3]);
    size_t n = rays.size() / 6;
    MTRandom rnd(atoi(argv[5]));
    FILE* f = wopen(argv[4]);
    for (size_t k = 0; k < n; k++) {
      Ray ray(Vector3d(rays[6 * k], rays[6 * k + 1], rays[6 * k + 2]),
              Vector3d(rays[6 * k + 3], rays[6 * k + 4], rays[6 * k + 5]));
      Spectrum v = radiance(0, env, ray, &rnd, 0, D_LINE_WAVELENGTH_SODIUM,
                            env->nextEventEstimation, env->participatingMedia);
      double c[3] = {v.x, v.y, v.z};
      fwrite(c, 8, 3, f);
    }
    fclose(f);
    return 0;
  }
  if (cmd == "hdr" && argc >= 5) {
    SceneEnv* env = load(argv[2]);
    Render r(*env);
    std::vector<double> img = read_f64(argv[3]);
    const int w = env->image_width, h = env->image_height;
    if ((int64_t)img.size() != (int64_t)w * h * 3) { fprintf(stderr, "image size mismatch\n"); return 3; }
    // Run() allocates the image (render.h:1142); here it is given
    struct RenderView { SceneEnv* env_p; Color* image; };
    Color* image = new Color[(size_t)w * h];
    for (int i = 0; i < w * h; i++) image[i] = Color(img[3 * i], img[3 * i + 1], img[3 * i + 2]);
    reinterpret_cast<RenderView*>(&r)->image = image;
    r.OutputHdr(argv[4]);
    return 0;
  }
  fprintf(stderr, "bad command\n");
  return 2;
}
