// sepx_sepio.cu -- SEP regular datasets (a text header "name.H" of key=value
// pairs plus a binary file named by its in= key), the on-disk format of the
// reference's inputs and outputs, read into and written from device vectors.
//
// The reference reaches these files through SEPlib (Born/sreg.cpp,
// Born/sregf.cpp: tag_init, read_axis, get_int/get_float/get_string,
// read_all/write_all, read_slice/write_slice); SEPlib is not part of this
// library, so the published conventions are implemented here directly:
//  * header: whitespace-separated key=value pairs, values optionally in
//    single or double quotes; a key given again overrides the earlier value
//    (headers grow by appending); words without '=' are ignored;
//  * axes: n1.. (missing: 1), o1.. (0), d1.. (1), label1.. (""); the number of
//    axes is the largest i with n_i given and n_i > 1 (at least 1);
//  * data: esize=4, data_format="xdr_float" (big-endian IEEE single, the SEP
//    default) or "native_float" (little-endian on every host this library
//    is compiled for), axis 1 fastest; in= is the data file (a relative path is looked
//    up beside the header first, then from the working directory; written
//    headers name the data file by its absolute path).
// Device transfers go through two pinned staging buffers on the library's
// stream; the big-endian byte swap runs on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/sepx.h"
#include "../../include/sepx_sepio.h"
#include "sepx_common.h"

namespace sepx {
namespace {

constexpr int kSepMaxAxes = SEPX_SEP_MAX_AXES;

__global__ void bswap32_kernel(uint32_t *p, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const uint32_t v = p[i];
    p[i] = __byte_perm(v, 0, 0x0123);
  }
}

void bswap_host(uint32_t *p, size_t n) {
  for (size_t i = 0; i < n; i++) {
    const uint32_t v = p[i];
    p[i] = (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
  }
}

bool host_is_little() {
  const uint32_t one = 1;
  unsigned char b;
  memcpy(&b, &one, 1);
  return b == 1;
}

struct Header {
  std::map<std::string, std::string> kv;
  std::string path, dir;
};

int parse_header(const char *path, Header *h) {
  FILE *f = fopen(path, "rb");
  if (!f) return set_error("sep: cannot open header %s: %s", path, strerror(errno));
  std::string txt;
  char buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, f)) > 0) txt.append(buf, got);
  fclose(f);
  h->path = path;
  const size_t slash = h->path.find_last_of('/');
  h->dir = slash == std::string::npos ? std::string(".") : h->path.substr(0, slash);
  size_t i = 0;
  const size_t n = txt.size();
  auto is_space = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; };
  while (i < n) {
    while (i < n && is_space(txt[i])) i++;
    size_t k0 = i;
    while (i < n && !is_space(txt[i]) && txt[i] != '=') i++;
    if (i >= n || txt[i] != '=' || i == k0) {   // a word without '='
      while (i < n && !is_space(txt[i])) i++;
      continue;
    }
    std::string key = txt.substr(k0, i - k0);
    i++;   // '='
    std::string val;
    if (i < n && (txt[i] == '"' || txt[i] == '\'')) {
      const char q = txt[i++];
      const size_t v0 = i;
      while (i < n && txt[i] != q) i++;
      val = txt.substr(v0, i - v0);
      if (i < n) i++;
    } else {
      const size_t v0 = i;
      while (i < n && !is_space(txt[i])) i++;
      val = txt.substr(v0, i - v0);
    }
    h->kv[key] = val;
  }
  return 0;
}

const std::string *find(const Header &h, const std::string &k) {
  auto it = h.kv.find(k);
  return it == h.kv.end() ? nullptr : &it->second;
}

struct Layout {
  int ndim = 1;
  int n[kSepMaxAxes];
  float o[kSepMaxAxes], d[kSepMaxAxes];
  long long n123 = 1;
  bool xdr = true;
  std::string data;
};

int layout_of(const Header &h, Layout *L) {
  L->ndim = 1;
  for (int a = 0; a < kSepMaxAxes; a++) {
    const std::string s = std::to_string(a + 1);
    const std::string *nv = find(h, "n" + s), *ov = find(h, "o" + s), *dv = find(h, "d" + s);
    if (nv) {
      char *end = nullptr;
      const long long v = strtoll(nv->c_str(), &end, 10);
      if (end == nv->c_str() || v < 1 || v > INT_MAX)
        return set_error("sep: %s: n%d=%s", h.path.c_str(), a + 1, nv->c_str());
      L->n[a] = (int)v;
    } else {
      L->n[a] = 1;
    }
    L->o[a] = ov ? strtof(ov->c_str(), nullptr) : 0.f;
    L->d[a] = dv ? strtof(dv->c_str(), nullptr) : 1.f;
    if (L->n[a] < 1) return set_error("sep: %s: n%d=%d", h.path.c_str(), a + 1, L->n[a]);
    if (nv && L->n[a] > 1) L->ndim = a + 1;
  }
  L->n123 = 1;
  for (int a = 0; a < kSepMaxAxes; a++) {
    if (L->n123 > (1LL << 60) / L->n[a])   // n[a] >= 1 here
      return set_error("sep: %s: the axes hold more than 2^60 elements", h.path.c_str());
    L->n123 *= L->n[a];
  }
  const std::string *es = find(h, "esize");
  if (es && atoi(es->c_str()) != 4)
    return set_error("sep: %s: esize=%s (only 4-byte floats are read)", h.path.c_str(), es->c_str());
  const std::string *fm = find(h, "data_format");
  if (!fm || *fm == "xdr_float") L->xdr = true;
  else if (*fm == "native_float") L->xdr = !host_is_little();
  else return set_error("sep: %s: data_format=%s is not a float format", h.path.c_str(), fm->c_str());
  const std::string *in = find(h, "in");
  if (!in || in->empty()) return set_error("sep: %s has no in= data file", h.path.c_str());
  L->data = *in;
  if (L->data[0] != '/') {
    const std::string beside = h.dir + "/" + L->data;
    FILE *t = fopen(beside.c_str(), "rb");
    if (t) {
      fclose(t);
      L->data = beside;
    }
  }
  return 0;
}

int open_layout(const char *header, Header *h, Layout *L) {
  if (!header) return set_error("sep: header path is NULL");
  if (int r = parse_header(header, h)) return r;
  return layout_of(*h, L);
}

// Two pinned staging buffers, reused across calls.
struct Staging {
  static constexpr size_t kBytes = size_t(32) << 20;
  void *buf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int ensure() {
    for (int i = 0; i < 2; i++) {
      if (!buf[i] && cudaMallocHost(&buf[i], kBytes) != cudaSuccess)
        return set_error("sep: cannot allocate pinned staging memory");
      if (!done[i] && cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) != cudaSuccess)
        return set_error("sep: cannot create an event");
    }
    return 0;
  }
};
Staging g_stage;

// Read `count` floats starting at element `first` of the data file into dst
// (host or device); byte order fixed on the way.
int read_span(FILE *f, const Layout &L, long long first, long long count, float *dst, bool dev,
              cudaStream_t st) {
  if (fseeko(f, (off_t)first * 4, SEEK_SET) != 0)
    return set_error("sep: seek failed in %s", L.data.c_str());
  if (!dev) {
    if (fread(dst, 4, (size_t)count, f) != (size_t)count)
      return set_error("sep: %s is shorter than its header says", L.data.c_str());
    if (L.xdr) bswap_host(reinterpret_cast<uint32_t *>(dst), (size_t)count);
    return 0;
  }
  if (int r = g_stage.ensure()) return r;
  const long long per = (long long)(Staging::kBytes / 4);
  int k = 0;
  for (long long done = 0; done < count; done += per, k ^= 1) {
    const long long c = std::min(per, count - done);
    if (cudaEventSynchronize(g_stage.done[k]) != cudaSuccess) return set_error("sep: event wait failed");
    if (fread(g_stage.buf[k], 4, (size_t)c, f) != (size_t)c)
      return set_error("sep: %s is shorter than its header says", L.data.c_str());
    float *d = dst + done;
    if (cudaMemcpyAsync(d, g_stage.buf[k], (size_t)c * 4, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return set_error("sep: host-to-device copy failed");
    if (cudaEventRecord(g_stage.done[k], st) != cudaSuccess) return set_error("sep: event record failed");
    if (L.xdr) {
      const int grid = (int)std::min<long long>((c + 255) / 256, 4096);
      bswap32_kernel<<<grid, 256, 0, st>>>(reinterpret_cast<uint32_t *>(d), c);
      if (cudaGetLastError() != cudaSuccess) return set_error("sep: byte-swap launch failed");
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return set_error("sep: stream synchronize failed");
  return 0;
}

int write_span(FILE *f, const float *src, long long count, bool xdr, bool dev, cudaStream_t st) {
  if (!dev) {
    std::vector<uint32_t> tmp;
    const long long per = 1 << 20;
    for (long long done = 0; done < count; done += per) {
      const long long c = std::min(per, count - done);
      tmp.assign(reinterpret_cast<const uint32_t *>(src + done),
                 reinterpret_cast<const uint32_t *>(src + done) + c);
      if (xdr) bswap_host(tmp.data(), tmp.size());
      if (fwrite(tmp.data(), 4, (size_t)c, f) != (size_t)c) return set_error("sep: write failed");
    }
    return 0;
  }
  if (int r = g_stage.ensure()) return r;
  const long long per = (long long)(Staging::kBytes / 4);
  for (long long done = 0; done < count; done += per) {
    const long long c = std::min(per, count - done);
    if (cudaMemcpyAsync(g_stage.buf[0], src + done, (size_t)c * 4, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return set_error("sep: device-to-host copy failed");
    if (xdr) bswap_host(reinterpret_cast<uint32_t *>(g_stage.buf[0]), (size_t)c);
    if (fwrite(g_stage.buf[0], 4, (size_t)c, f) != (size_t)c) return set_error("sep: write failed");
  }
  return 0;
}

cudaStream_t lib_stream(bool dev, int *rc) {
  *rc = 0;
  if (!dev) return nullptr;
  void *s = sepx_get_stream();
  if (!s) *rc = set_error("sep: setup_cuda must be called before device transfers");
  return static_cast<cudaStream_t>(s);
}

}  // namespace
}  // namespace sepx

using namespace sepx;

extern "C" {

int sepx_sep_info(const char *header, int *ndim, int n[8], float o[8], float d[8]) {
  Header h;
  Layout L;
  if (int r = open_layout(header, &h, &L)) return r;
  if (ndim) *ndim = L.ndim;
  for (int a = 0; a < kSepMaxAxes; a++) {
    if (n) n[a] = L.n[a];
    if (o) o[a] = L.o[a];
    if (d) d[a] = L.d[a];
  }
  return 0;
}

int sepx_sep_par(const char *header, const char *key, char *out, int cap) {
  Header h;
  if (!header || !key || !out || cap < 1) return set_error("sep_par: invalid arguments");
  if (int r = parse_header(header, &h)) return r;
  const std::string *v = find(h, key);
  if (!v) return 1;   // not given (no error recorded)
  if ((int)v->size() + 1 > cap) return set_error("sep_par: value of %s is longer than %d", key, cap - 1);
  memcpy(out, v->c_str(), v->size() + 1);
  return 0;
}

int sepx_sep_read(const char *header, long long first, long long count, float *dst, int on_device) {
  Header h;
  Layout L;
  if (int r = open_layout(header, &h, &L)) return r;
  if (!dst || first < 0 || count < 0 || first > L.n123 || count > L.n123 - first)
    return set_error("sep_read: %lld elements from %lld do not lie inside the %lld of %s", count,
                     first, L.n123, header);
  int rc;
  cudaStream_t st = lib_stream(on_device != 0, &rc);
  if (rc) return rc;
  FILE *f = fopen(L.data.c_str(), "rb");
  if (!f) return set_error("sep_read: cannot open %s: %s", L.data.c_str(), strerror(errno));
  rc = count ? read_span(f, L, first, count, dst, on_device != 0, st) : 0;
  fclose(f);
  return rc;
}

int sepx_sep_read_window(const char *header, const int *nw, const int *fw, const int *jw, float *dst,
                         int on_device) {
  Header h;
  Layout L;
  if (int r = open_layout(header, &h, &L)) return r;
  if (!nw || !dst) return set_error("sep_read_window: invalid arguments");
  int N[kSepMaxAxes], F[kSepMaxAxes], J[kSepMaxAxes];
  long long total = 1;
  for (int a = 0; a < kSepMaxAxes; a++) {
    N[a] = nw[a];
    F[a] = fw ? fw[a] : 0;
    J[a] = jw ? jw[a] : 1;
    if (N[a] < 1 || F[a] < 0 || J[a] < 1 || F[a] + (long long)(N[a] - 1) * J[a] >= L.n[a])
      return set_error("sep_read_window: axis %d window n=%d f=%d j=%d outside n=%d", a + 1, N[a],
                       F[a], J[a], L.n[a]);
    total *= N[a];
  }
  int rc;
  cudaStream_t st = lib_stream(on_device != 0, &rc);
  if (rc) return rc;
  FILE *f = fopen(L.data.c_str(), "rb");
  if (!f) return set_error("sep_read_window: cannot open %s: %s", L.data.c_str(), strerror(errno));
  // rows along axis 1 are read whole (strided rows pick every J[0]-th sample)
  const long long span = (long long)(N[0] - 1) * J[0] + 1;
  std::vector<float> row((size_t)span), out((size_t)N[0]);
  std::vector<float> host;
  if (on_device) host.resize((size_t)std::max<long long>(N[0], std::min<long long>(total, 1 << 22)));
  long long w = 0, hfill = 0;
  long long stride[kSepMaxAxes];
  stride[0] = 1;
  for (int a = 1; a < kSepMaxAxes; a++) stride[a] = stride[a - 1] * L.n[a - 1];
  const long long nrows = total / N[0];
  int idx[kSepMaxAxes] = {0};
  for (long long r = 0; r < nrows && rc == 0; r++) {
    long long off = F[0];
    for (int a = 1; a < kSepMaxAxes; a++) off += (long long)(F[a] + idx[a] * J[a]) * stride[a];
    rc = read_span(f, L, off, span, row.data(), false, nullptr);
    if (rc) break;
    for (int i = 0; i < N[0]; i++) out[i] = row[(size_t)i * J[0]];
    if (!on_device) {
      memcpy(dst + w, out.data(), sizeof(float) * N[0]);
    } else {
      if (hfill + N[0] > (long long)host.size()) {
        if (cudaMemcpyAsync(dst + w - hfill, host.data(), hfill * 4, cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
          rc = set_error("sep_read_window: host-to-device copy failed");
        hfill = 0;
      }
      memcpy(host.data() + hfill, out.data(), sizeof(float) * N[0]);
      hfill += N[0];
    }
    w += N[0];
    for (int a = 1; a < kSepMaxAxes; a++) {
      if (++idx[a] < N[a]) break;
      idx[a] = 0;
    }
  }
  if (rc == 0 && on_device && hfill > 0) {
    if (cudaMemcpyAsync(dst + w - hfill, host.data(), hfill * 4, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = set_error("sep_read_window: host-to-device copy failed");
  }
  fclose(f);
  return rc;
}

int sepx_sep_write(const char *header, int ndim, const int *n, const float *o, const float *d,
                   const char *labels, const float *src, int on_device, int xdr) {
  if (!header || !n || ndim < 1 || ndim > kSepMaxAxes || !src)
    return set_error("sep_write: invalid arguments");
  long long total = 1;
  for (int a = 0; a < ndim; a++) {
    if (n[a] < 1) return set_error("sep_write: n%d=%d", a + 1, n[a]);
    total *= n[a];
  }
  int rc;
  cudaStream_t st = lib_stream(on_device != 0, &rc);
  if (rc) return rc;
  const std::string hp = header, dp = hp + "@";
  std::vector<std::string> lab;
  if (labels) {
    std::string s = labels;
    size_t p = 0;
    while (p <= s.size()) {
      const size_t q = s.find('\n', p);
      lab.push_back(s.substr(p, q == std::string::npos ? std::string::npos : q - p));
      if (q == std::string::npos) break;
      p = q + 1;
    }
  }
  FILE *f = fopen(dp.c_str(), "wb");
  if (!f) return set_error("sep_write: cannot create %s: %s", dp.c_str(), strerror(errno));
  rc = write_span(f, src, total, xdr != 0 ? true : !host_is_little(), on_device != 0, st);
  if (fclose(f) != 0 && rc == 0) rc = set_error("sep_write: closing %s failed", dp.c_str());
  if (rc) return rc;
  FILE *h = fopen(hp.c_str(), "wb");
  if (!h) return set_error("sep_write: cannot create %s: %s", hp.c_str(), strerror(errno));
  for (int a = 0; a < ndim; a++) {
    fprintf(h, "n%d=%d o%d=%.9g d%d=%.9g", a + 1, n[a], a + 1, o ? (double)o[a] : 0.0, a + 1,
            d ? (double)d[a] : 1.0);
    if (a < (int)lab.size() && !lab[a].empty()) fprintf(h, " label%d=\"%s\"", a + 1, lab[a].c_str());
    fprintf(h, "\n");
  }
  char full[4096];
  const std::string absdata = realpath(dp.c_str(), full) ? std::string(full) : dp;
  fprintf(h, "esize=4 data_format=\"%s\"\nin=\"%s\"\n", xdr ? "xdr_float" : "native_float",
          absdata.c_str());
  if (fclose(h) != 0) return set_error("sep_write: closing %s failed", hp.c_str());
  return 0;
}

}  // extern "C"
