// C++ user of the operator API on the GPU (tests/test_gpu_dataimg.py builds
// and runs it): image_rtm_3d, data_rtm_3d and tmute on device vectors.  Reads
// float32 inputs from <dir>/<name>.bin, writes the results beside them.
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sepx.h"
#include "sepx_ops.h"

static std::string g_dir;

static std::vector<float> load(const char *name, size_t n) {
  std::vector<float> v(n);
  FILE *f = fopen((g_dir + "/" + name + ".bin").c_str(), "rb");
  if (!f || fread(v.data(), sizeof(float), n, f) != n) throw std::runtime_error(name);
  fclose(f);
  return v;
}

static void save(const char *name, const hypercube_float &h) {
  std::vector<float> v((size_t)h.n123);
  h.download(v.data());
  FILE *f = fopen((g_dir + "/" + name + ".bin").c_str(), "wb");
  if (!f || fwrite(v.data(), sizeof(float), v.size(), f) != v.size()) throw std::runtime_error(name);
  fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  g_dir = argv[1];
  try {
    if (sepx_setup_cuda(1)) throw std::runtime_error(sepx_last_error());
    // image on (9, 7, 6) cells of (10, 12.5, 5) m; a 6 x 5 x 4 window at `so`
    const std::vector<float> so = load("so", 3);
    image_rtm_3d im({axis(9, 0.f, 10.f), axis(7, 0.f, 12.5f), axis(6, 0.f, 5.f)});
    im.image->upload(load("img", 9 * 7 * 6).data());
    hypercube_float sub({axis(6, so[0], 10.f), axis(5, so[1], 12.5f), axis(4, so[2], 5.f)});
    sub.upload(load("sub", 6 * 5 * 4).data());
    im.add_image(&sub);
    save("out_add", *im.image);
    hypercube_float mute(im.image->axes);
    mute.upload(load("mute", 9 * 7 * 6).data());
    im.set_mute(mute);
    std::unique_ptr<hypercube_float> ex(im.extract_sub(sub.get_axis(1), sub.get_axis(2), sub.get_axis(3)));
    save("out_sub", *ex);
    im.write_volume();
    save("out_muted", *im.image);

    // data of 3 shots, (t 50, x 4, y 2); shot 1 accumulated twice
    data_rtm_3d dat({axis(50, 0.f, .004f), axis(4), axis(2), axis(3)});
    dat.upload(load("all", 50 * 4 * 2 * 3).data());
    hypercube_float shot({axis(50, 0.f, .004f), axis(4), axis(2)});
    shot.upload(load("shot", 50 * 4 * 2).data());
    dat.add_data(1, &shot);
    dat.add_data(1, &shot);
    save("out_data", dat);

    // tmute: traces (t 64 of 4 ms, x 6 of 25 m from 50 m, 3 cubes, 2 shots)
    const std::vector<axis> ta = {axis(64, 0.f, .004f), axis(6, 50.f, 25.f), axis(3), axis(2)};
    hypercube_float m(ta), d(ta);
    m.upload(load("tm_model", 64 * 6 * 6).data());
    d.upload(load("tm_data", 64 * 6 * 6).data());
    tmute op(0.04f, 1800.f, &m, &d);
    op.forward(false, &m, &d);   // d = T m
    save("out_tm_fwd", d);
    d.upload(load("tm_data", 64 * 6 * 6).data());
    op.adjoint(true, &m, &d);    // m += T' d
    save("out_tm_adj", m);
    if (sepx_synchronize()) throw std::runtime_error(sepx_last_error());
  } catch (const std::exception &e) {
    fprintf(stderr, "dataimg_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
