// A C++ caller of the operator API written the way the reference's
// least-squares RTM program is (Born/RTM_inv.cpp:14-68): parameters, data,
// wavelet with its shot axes, velocity, zeroed image, rtm_zero_op through
// the reference's constructor, simple_solver with cgstep, solve(niter),
// return_model added into the image.  SEP files are replaced by raw float32
// files in <dir> (tests/test_gpu_rtm_inv.py writes them and runs this).
//
//   dims.bin: m1 m2 m3 d nt dt rnx rny ro2 rd2 ro3 rd3 nsx osx dsx nsy osy dsy
//             src_depth nbound bc_a bc_b niter nwav dtw
//   vel.bin, wavelet.bin, data.bin  ->  model.bin, resid.bin (float64)
#include <cstdio>
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

static void save(const char *name, const void *p, size_t bytes) {
  FILE *f = fopen((g_dir + "/" + name + ".bin").c_str(), "wb");
  if (!f || fwrite(p, 1, bytes, f) != bytes) throw std::runtime_error(name);
  fclose(f);
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  g_dir = argv[1];
  try {
    const std::vector<float> D = load("dims", 25);
    int k = 0;
    const int m1 = (int)D[k++], m2 = (int)D[k++], m3 = (int)D[k++];
    const float d = D[k++];
    const int nt = (int)D[k++];
    const float dt = D[k++];
    const int rnx = (int)D[k++], rny = (int)D[k++];
    const float ro2 = D[k++], rd2 = D[k++], ro3 = D[k++], rd3 = D[k++];
    const int nsx = (int)D[k++];
    const float osx = D[k++], dsx = D[k++];
    const int nsy = (int)D[k++];
    const float osy = D[k++], dsy = D[k++];
    const float src_depth = D[k++];
    const int nbound = (int)D[k++];
    const float bc_a = D[k++], bc_b = D[k++];
    const int niter_arg = (int)D[k++], nwav = (int)D[k++];
    const float dtw = D[k++];

    param_func pars;
    pars.set("bc_a", bc_a).set("bc_b", bc_b).set("nbound", nbound).set("niter", niter_arg)
        .set("src_depth", src_depth).set("rec_depth", 0.0).set("n_gpus", 1).set("aper", 8.0);

    data_rtm_3d data({axis(nt, 0.f, dt), axis(rnx, ro2, rd2), axis(rny, ro3, rd3),
                      axis(nsx, osx, dsx), axis(nsy, osy, dsy)}, &pars);
    data.upload(load("data", (size_t)data.n123).data());
    source_func wavelet(axis(nwav, 0.f, dtw), load("wavelet", nwav).data());
    axis asx = data.get_axis(4);
    axis asy = data.get_axis(5);
    int niter = pars.get_int("niter", 5);
    float sdepth = pars.get_float("src_depth", 0.);
    wavelet.set_sources_3d(sdepth, asx, asy);
    const std::vector<float> v = load("vel", (size_t)m1 * m2 * m3);
    vel_fd_3d vel({axis(m1, 0.f, d), axis(m2, 0.f, d), axis(m3, 0.f, d)}, v.data());
    image_rtm_3d image("image", &vel);
    image.zero();

    int n_gpus = pars.get_int("n_gpus", 0);
    if (sepx_setup_cuda(n_gpus)) throw std::runtime_error(sepx_last_error());

    float aper = pars.get_float("aper", 8.);
    int *rand_vec = 0;
    bool encode = false;
    rtm_zero_op op(&pars, &vel, &wavelet, &data, &image, aper, false, encode, rand_vec, true, false);

    cgstep *st = new cgstep();
    simple_solver *solv = new simple_solver(st, &data, &op);
    solv->set_verbose(0);
    solv->solve(niter);

    hypercube_float *mine = (hypercube_float *)solv->return_model();
    image.add(mine);

    std::vector<float> out((size_t)image.image->n123);
    image.image->download(out.data());
    save("model", out.data(), out.size() * sizeof(float));
    save("resid", solv->resid.data(), solv->resid.size() * sizeof(double));
    delete mine;
    delete solv;
    delete st;
  } catch (const std::exception &e) {
    fprintf(stderr, "rtm_inv_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
