// In-memory stand-ins for the SEPlib calls made by the reference's host C++,
// so that its classes (vel_fd_3d, source_func, data_rtm_3d, image_rtm_3d,
// oc_float, rtm_zero_op, ...) run unchanged inside the oracle's reference library
// oracle/_ref/libsepref.so.  A "file" is a named byte buffer with a cursor and
// SEP-style axes; parameters are a name->string table.  Test infrastructure.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "seplib.h"

namespace {
struct RefFile {
  std::vector<char> data;
  long pos = 0;
  std::vector<int> n;
  std::vector<float> o, d;
};
std::map<std::string, RefFile> g_files;
std::map<std::string, std::string> g_params;

RefFile &file(const char *tag) { return g_files[std::string(tag)]; }

int parse(const std::string &v, const char *type, void *val) {
  if (!strcmp(type, "d") || !strcmp(type, "i")) {
    *(int *)val = atoi(v.c_str());
  } else if (!strcmp(type, "f") || !strcmp(type, "r")) {
    *(float *)val = (float)atof(v.c_str());
  } else if (!strcmp(type, "s")) {
    strcpy((char *)val, v.c_str());
  } else {
    return 0;
  }
  return 1;
}
}  // namespace

extern "C" {

int seperr(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  fprintf(stderr, "seperr: ");
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  fflush(stderr);
  abort();
}

int sreed(const char *tag, void *buf, int nbytes) {
  RefFile &f = file(tag);
  long avail = (long)f.data.size() - f.pos;
  if (avail < 0) avail = 0;
  long take = nbytes < avail ? nbytes : avail;
  if (take > 0) memcpy(buf, f.data.data() + f.pos, (size_t)take);
  if (take < nbytes) memset((char *)buf + take, 0, (size_t)(nbytes - take));
  f.pos += nbytes;
  return nbytes;
}

int srite(const char *tag, void *buf, int nbytes) {
  RefFile &f = file(tag);
  if ((long)f.data.size() < f.pos + nbytes) f.data.resize((size_t)(f.pos + nbytes), 0);
  memcpy(f.data.data() + f.pos, buf, (size_t)nbytes);
  f.pos += nbytes;
  return nbytes;
}

int sseek(const char *tag, int off, int whence) {
  RefFile &f = file(tag);
  if (whence == 0) f.pos = off;
  else if (whence == 1) f.pos += off;
  else f.pos = (long)f.data.size() + off;
  return (int)f.pos;
}

int sseek_block(const char *tag, int block, int blocksize, int whence) {
  RefFile &f = file(tag);
  long off = (long)block * (long)blocksize;
  if (whence == 0) f.pos = off;
  else if (whence == 1) f.pos += off;
  else f.pos = (long)f.data.size() + off;
  return 0;
}

int getch(const char *name, const char *type, void *val) {
  auto it = g_params.find(name);
  if (it == g_params.end()) return 0;
  return parse(it->second, type, val);
}

int putch(const char *, const char *, void *) { return 0; }

int auxpar(const char *name, const char *type, void *val, const char *tag) {
  auto it = g_params.find(std::string(tag) + ":" + name);
  if (it == g_params.end()) return 0;
  return parse(it->second, type, val);
}

int auxputch(const char *, const char *, void *, const char *) { return 0; }
FILE *auxinout(const char *tag) { (void)file(tag); return stderr; }
FILE *auxin(const char *tag) { (void)file(tag); return stderr; }
FILE *auxout(const char *tag) { (void)file(tag); return stderr; }
int auxclose(const char *) { return 0; }

int sreed_window(const char *, int *, int *, int *, int *, int *, int, void *) {
  return seperr("sreed_window is not available in the oracle's reference library\n");
}
int srite_window(const char *, int *, int *, int *, int *, int *, int, void *) {
  return seperr("srite_window is not available in the oracle's reference library\n");
}

int sep_get_number_data_axes(const char *tag, int *n) {
  auto it = g_files.find(tag);
  if (it == g_files.end() || it->second.n.empty()) return 1;
  *n = (int)it->second.n.size();
  return 0;
}

int sep_get_data_axis_par(const char *tag, int *i, int *n, float *o, float *d, char *label) {
  RefFile &f = file(tag);
  int k = *i - 1;
  if (k >= 0 && k < (int)f.n.size()) {
    *n = f.n[k]; *o = f.o[k]; *d = f.d[k];
  } else {
    *n = 1; *o = 0.f; *d = 1.f;
  }
  if (label) strcpy(label, "none");
  return 0;
}

int sep_put_data_axis_par(const char *tag, int *i, int *n, float *o, float *d, char *) {
  RefFile &f = file(tag);
  int k = *i - 1;
  if (k < 0) return 1;
  if ((int)f.n.size() <= k) { f.n.resize(k + 1, 1); f.o.resize(k + 1, 0.f); f.d.resize(k + 1, 1.f); }
  f.n[k] = *n; f.o[k] = *o; f.d[k] = *d;
  return 0;
}

void initpar(int, char **) {}

// oc_float::make_temp (Born/oc_float.cpp:406-412) names temporary datasets
// with mkstemp, which would create files in the working directory: the
// oracle's datasets live in memory, so this library's own calls get a
// unique name and no file (no descriptor is returned; the reference ignores it).
int mkstemp(char *tmpl) {
  static unsigned long long counter = 0;
  const size_t n = strlen(tmpl);
  unsigned long long v = ++counter;
  for (size_t i = n; i > 0 && tmpl[i - 1] == 'X'; i--, v /= 10) tmpl[i - 1] = (char)('0' + v % 10);
  return -1;
}

// ---- registry access for the oracle ----
void ref_reset(void) { g_files.clear(); g_params.clear(); }

void ref_file_put(const char *tag, int ndim, const int *n, const float *o, const float *d,
                  const void *data, long nbytes) {
  RefFile &f = g_files[std::string(tag)];
  f.n.assign(n, n + ndim);
  f.o.assign(o, o + ndim);
  f.d.assign(d, d + ndim);
  f.data.assign((const char *)data, (const char *)data + nbytes);
  f.pos = 0;
}

long ref_file_size(const char *tag) {
  auto it = g_files.find(tag);
  return it == g_files.end() ? -1 : (long)it->second.data.size();
}

long ref_file_get(const char *tag, void *out, long nbytes) {
  auto it = g_files.find(tag);
  if (it == g_files.end()) return -1;
  long take = (long)it->second.data.size();
  if (take > nbytes) take = nbytes;
  memcpy(out, it->second.data.data(), (size_t)take);
  return take;
}

void ref_param_put(const char *name, const char *value) { g_params[name] = value; }

}  // extern "C"
