/* Forced-include shim that lets the reference's MSVC-era sources compile with
 * g++ on Linux.  Test infrastructure only: it is used by oracle/build_ref.sh
 * to build the reference renderer as a checker, never by the product. */
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <strings.h>
#include <string>
#define __declspec(x) __attribute__((aligned(16)))
#ifndef _MAX_PATH
#define _MAX_PATH 1024
#define _MAX_DRIVE 16
#define _MAX_DIR 1024
#define _MAX_FNAME 512
#define _MAX_EXT 64
#endif
#define strcmpi strcasecmp
static inline void* _aligned_malloc(size_t n, size_t a) {
  void* p = nullptr;
  if (posix_memalign(&p, a < sizeof(void*) ? sizeof(void*) : a, n)) return nullptr;
  return p;
}
static inline void _aligned_free(void* p) { free(p); }
/* POSIX stand-in for the MSVC path splitter (drive is always empty). */
static inline void _splitpath(const char* path, char* drive, char* dir, char* fname, char* ext) {
  std::string s(path ? path : "");
  if (drive) drive[0] = '\0';
  size_t slash = s.find_last_of("/\\");
  std::string d = (slash == std::string::npos) ? "" : s.substr(0, slash + 1);
  std::string f = (slash == std::string::npos) ? s : s.substr(slash + 1);
  size_t dot = f.find_last_of('.');
  std::string e = (dot == std::string::npos) ? "" : f.substr(dot);
  if (dot != std::string::npos) f = f.substr(0, dot);
  if (dir) strcpy(dir, d.c_str());
  if (fname) strcpy(fname, f.c_str());
  if (ext) strcpy(ext, e.c_str());
}

/* Read-only probe of the Kerr trace loop (scene.cpp:554-688): the build
 * recipe inserts one statement that copies the loop state into this record,
 * so the harness can report the final Boyer-Lindquist state and the polyline
 * direction.  It does not change what the loop computes. */
struct KerrProbe {
  int reached_end = 0;
  int steps = 0;
  double y[6] = {0, 0, 0, 0, 0, 0};
  double org[3] = {0, 0, 0};
  double dir[3] = {0, 0, 0};
};
extern thread_local KerrProbe prender_kerr_probe;
#define PRENDER_KERR_PROBE(END, CNT, Y, ORG, DIR)                                  \
  do {                                                                             \
    prender_kerr_probe.reached_end = (END);                                        \
    prender_kerr_probe.steps = (CNT);                                              \
    for (int q_ = 0; q_ < 6; q_++) prender_kerr_probe.y[q_] = (Y)[q_];             \
    prender_kerr_probe.org[0] = (ORG).x; prender_kerr_probe.org[1] = (ORG).y;      \
    prender_kerr_probe.org[2] = (ORG).z;                                           \
    prender_kerr_probe.dir[0] = (DIR).x; prender_kerr_probe.dir[1] = (DIR).y;      \
    prender_kerr_probe.dir[2] = (DIR).z;                                           \
  } while (0)
