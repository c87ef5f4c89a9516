// e3d_run -- command-line driver mirroring the reference's `program elas3d`
// (src/elas3dxtal_pcg.f90:186-552) on the GB300 library: read (or generate) a
// microstructure, femat, affine guess, energy, PCG, energy, averaged stress,
// full-field stress and von Mises, with the reference's text outputs:
//   output_SS316L_polycrystal.txt   run log (:278-537)
//   cg_history_polycrystal.txt      energy and rel_res per solve (:466-492)
//   cgitr_SS316L_polycrystal.txt    rel_res per PCG iteration (:1458, :2019-2021)
//   fullfield_poly.h5               pix, vm, stress_tensor(ns,6) (:2840-2874)
// The microstructure comes from an HDF5 file with the datasets "pix" and
// "orientation" (input_structure_poly.h5, read as ppixel_hdf5 reads it,
// :2879-2990), from a .e3d container, or from the built-in generator.
// Run `e3d_run --help` for the options.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "e3d_gpu.h"
#include "e3d_micro.h"

namespace {

void usage() {
  std::printf(
      "usage: e3d_run [options]\n"
      "  --input FILE              microstructure: HDF5 (\"pix\", \"orientation\"; grid from the\n"
      "                            \"dimensions\" attribute or --grid) or .e3d\n"
      "  --grid NX NY NZ           grid of an HDF5 input without a \"dimensions\" attribute\n"
      "  --generate N NGRAINS SEED PORE_FRAC   periodic Voronoi N^3 instead of --input\n"
      "  --c11 P --c12 P --c44 P   cubic constants in Pa (206e9 133e9 119e9)\n"
      "  --strain exx eyy ezz exz eyz exy      tensor macro strain (0 0 1e-3 0 0 0)\n"
      "  --tol T --max-iter N      stop test (1e-8, 10000)\n"
      "  --precision fp64|mixed    arithmetic (fp64)\n"
      "  --criterion ref|precond   stop test sqrt(z.g/|g0|^2) or sqrt(z.g/z0.g0) (ref)\n"
      "  --cg                      unpreconditioned CG (applications/sec3_1/cg)\n"
      "  --isotropic E1 NU1        inclusion phase modulus / Poisson ratio (0 0)\n"
      "  --flag-m 0|1              0: isotropic matrix, 1: rotated cubic grains (1)\n"
      "  --outdir DIR              output directory (.)\n"
      "  --fullfield               also write fullfield_poly.h5\n"
      "  --json                    print one JSON metrics line for the solve on stdout\n"
      "  --checkpoint FILE         save the PCG state at exit (resume with --resume)\n"
      "  --resume FILE             continue a saved solve\n"
      "  --device N                CUDA device (0)\n");
}

int fail(const char* what, int rc) {
  std::fprintf(stderr, "e3d_run: %s: %s", what, e3d_strerror(rc));
  if (rc == E3D_ERR_CUDA) std::fprintf(stderr, " [%s]", e3d_last_cuda_error());
  std::fprintf(stderr, "\n");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  std::string input, outdir = ".", ckpt, resume;
  int gen_n = 0, gen_g = 0, grid[3] = {0, 0, 0};
  unsigned long long gen_seed = 1;
  double gen_pores = 0.0;
  double c11 = 206.0e9, c12 = 133.0e9, c44 = 119.0e9, e1 = 0.0, nu1 = 0.0;
  double strain[6] = {0, 0, 1.0e-3, 0, 0, 0};
  float tol = 1.0e-8f;
  int max_iter = 10000, precision = E3D_PREC_FP64, criterion = E3D_CRIT_REF, device = 0, flag_m = 1;
  int precond = E3D_PRECOND_BLOCK_JACOBI;
  bool fullfield = false, json = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto need = [&](int k) {
      if (i + k >= argc) {
        usage();
        std::exit(2);
      }
    };
    if (a == "--help" || a == "-h") {
      usage();
      return 0;
    } else if (a == "--input") {
      need(1);
      input = argv[++i];
    } else if (a == "--grid") {
      need(3);
      for (int k = 0; k < 3; ++k) grid[k] = std::atoi(argv[++i]);
      if (grid[0] < 1 || grid[1] < 1 || grid[2] < 1) {
        usage();
        return 2;
      }
    } else if (a == "--generate") {
      need(4);
      gen_n = std::atoi(argv[++i]);
      gen_g = std::atoi(argv[++i]);
      gen_seed = std::strtoull(argv[++i], nullptr, 10);
      gen_pores = std::atof(argv[++i]);
    } else if (a == "--c11") {
      need(1);
      c11 = std::atof(argv[++i]);
    } else if (a == "--c12") {
      need(1);
      c12 = std::atof(argv[++i]);
    } else if (a == "--c44") {
      need(1);
      c44 = std::atof(argv[++i]);
    } else if (a == "--strain") {
      need(6);
      for (int k = 0; k < 6; ++k) strain[k] = std::atof(argv[++i]);
    } else if (a == "--tol") {
      need(1);
      tol = (float)std::atof(argv[++i]);
    } else if (a == "--max-iter") {
      need(1);
      max_iter = std::atoi(argv[++i]);
    } else if (a == "--precision") {
      need(1);
      precision = std::strcmp(argv[++i], "mixed") == 0 ? E3D_PREC_MIXED : E3D_PREC_FP64;
    } else if (a == "--criterion") {
      need(1);
      criterion = std::strcmp(argv[++i], "precond") == 0 ? E3D_CRIT_PRECOND_REL : E3D_CRIT_REF;
    } else if (a == "--cg") {
      precond = E3D_PRECOND_NONE;
    } else if (a == "--isotropic") {
      need(2);
      e1 = std::atof(argv[++i]);
      nu1 = std::atof(argv[++i]);
    } else if (a == "--flag-m") {
      need(1);
      flag_m = std::atoi(argv[++i]);
    } else if (a == "--outdir") {
      need(1);
      outdir = argv[++i];
    } else if (a == "--json") {
      json = true;
    } else if (a == "--fullfield") {
      fullfield = true;
    } else if (a == "--checkpoint") {
      need(1);
      ckpt = argv[++i];
    } else if (a == "--resume") {
      need(1);
      resume = argv[++i];
    } else if (a == "--device") {
      need(1);
      device = std::atoi(argv[++i]);
    } else {
      std::fprintf(stderr, "e3d_run: unknown option %s\n", a.c_str());
      usage();
      return 2;
    }
  }
  // ---- microstructure (ppixel_hdf5, :380)
  int nx = 0, ny = 0, nz = 0, ng = 0;
  std::vector<int32_t> pix;
  std::vector<double> rod;
  bool is_h5 = false;
  if (!input.empty()) {
    if (FILE* f = std::fopen(input.c_str(), "rb")) {  // HDF5 format signature at 0 or after a user block
      unsigned char sig[8];
      for (long off = 0; !is_h5 && off <= 8192; off = off ? 2 * off : 512)
        if (std::fseek(f, off, SEEK_SET) == 0 && std::fread(sig, 1, 8, f) == 8 &&
            std::memcmp(sig, "\x89HDF\r\n\x1a\n", 8) == 0)
          is_h5 = true;
      std::fclose(f);
    }
  }
  if (is_h5) {
    int64_t npix = 0, nori = 0;
    int32_t dims[3] = {0, 0, 0};
    if (e3d_h5_micro_info(input.c_str(), &npix, &nori, dims) != 0) {
      std::fprintf(stderr, "e3d_run: %s: %s\n", input.c_str(), e3d_last_cuda_error());
      return 1;
    }
    if (grid[0] > 0) {
      nx = grid[0], ny = grid[1], nz = grid[2];
    } else if (dims[0] > 0 && dims[1] > 0 && dims[2] > 0) {
      nx = dims[0], ny = dims[1], nz = dims[2];
    } else {
      std::fprintf(stderr, "e3d_run: %s has no \"dimensions\" attribute; give --grid NX NY NZ\n", input.c_str());
      return 1;
    }
    if (nori % 3 != 0) {
      std::fprintf(stderr, "e3d_run: %s: orientation holds %lld values, not 3 per grain\n", input.c_str(),
                   (long long)nori);
      return 1;
    }
    ng = (int)(nori / 3);
    pix.resize((size_t)nx * ny * nz);
    rod.resize(3 * (size_t)std::max(ng, 1));
    if (e3d_h5_micro_read(input.c_str(), (int64_t)nx * ny * nz, ng, pix.data(), rod.data()) != 0) {
      std::fprintf(stderr, "e3d_run: %s\n", e3d_last_cuda_error());
      return 1;
    }
  } else if (!input.empty()) {
    if (e3d_micro_read_header(input.c_str(), &nx, &ny, &nz, &ng) != 0) {
      std::fprintf(stderr, "e3d_run: cannot read %s\n", input.c_str());
      return 1;
    }
    pix.resize((size_t)nx * ny * nz);
    rod.resize(3 * (size_t)ng);
    if (e3d_micro_read(input.c_str(), nx, ny, nz, ng, pix.data(), rod.data()) != 0) {
      std::fprintf(stderr, "e3d_run: %s: size or phase-range check failed\n", input.c_str());
      return 1;
    }
  } else if (gen_n > 0 && gen_g > 0) {
    nx = ny = nz = gen_n;
    ng = gen_g;
    pix.resize((size_t)nx * ny * nz);
    rod.resize(3 * (size_t)ng);
    if (e3d_micro_grains(nx, ny, nz, ng, 0.0, gen_seed, pix.data(), rod.data()) != 0) return 1;
    if (gen_pores > 0.0 && e3d_micro_spherical_pores(nx, ny, nz, gen_pores, std::log(3.0), 0.4, ng + 1,
                                                     gen_seed + 7919, pix.data()) < 0)
      return 1;
  } else {
    usage();
    return 2;
  }
  const long long ns = (long long)nx * ny * nz;
  const int nphase = ng + 1;
  const std::string out_path = outdir + "/output_SS316L_polycrystal.txt";
  FILE* out = std::fopen(out_path.c_str(), "w");
  if (!out) {
    std::fprintf(stderr, "e3d_run: cannot write %s\n", out_path.c_str());
    return 1;
  }
  const auto t_start = std::chrono::steady_clock::now();
  std::fprintf(out, "nx = %4d, ny =%4d, nz =%4d, ns =%12lld\n", nx, ny, nz, ns);
  std::printf("nx = %4d, ny =%4d, nz =%4d, ns =%12lld\n", nx, ny, nz, ns);
  // volume fractions (assig, :2410-2468)
  {
    std::vector<double> prob((size_t)nphase, 0.0);
    for (long long m = 0; m < ns; ++m) prob[(size_t)pix[(size_t)m] - 1] += 1.0;
    for (int i = 0; i < nphase; ++i)
      std::fprintf(out, "Volume fraction of phase %7d is %20.6f\n", i + 1, prob[(size_t)i] / (double)ns);
  }
  std::fprintf(out, " Applied engineering strains\n  exx eyy ezz exz eyz exy\n %g %g %g %g %g %g\n", strain[0],
               strain[1], strain[2], 2 * strain[3], 2 * strain[4], 2 * strain[5]);
  e3d_problem_t p;
  e3d_problem_defaults(&p, nx, ny, nz, nphase);
  p.c11 = c11;
  p.c12 = c12;
  p.c44 = c44;
  p.e1 = e1;
  p.nu1 = nu1;
  p.flag_m = flag_m;
  p.tol = tol;
  p.max_iter = max_iter;
  p.precision = precision;
  p.criterion = criterion;
  p.preconditioner = precond;
  p.device = device;
  if (precond == E3D_PRECOND_NONE) p.divergence_reset = 0;  // the CG variant has none
  for (int k = 0; k < 6; ++k) p.strain[k] = strain[k];
  e3d_handle_t* h = nullptr;
  int rc = e3d_create(&h, &p);
  if (rc) return fail("e3d_create", rc);
  if ((rc = e3d_upload(h, pix.data(), rod.data()))) return fail("e3d_upload", rc);
  if ((rc = e3d_femat(h))) return fail("e3d_femat", rc);  // :417
  double utot0 = 0.0, gg0 = 0.0;
  e3d_solve_stats_t st{};
  if (resume.empty()) {
    if ((rc = e3d_init_affine(h))) return fail("e3d_init_affine", rc);  // :423-438
    if ((rc = e3d_energy(h, &utot0, &gg0))) return fail("e3d_energy", rc);  // :449-453
    std::fprintf(out, " Initial energy= %.10e gg= %.10e\n", utot0, gg0);
    std::printf("Initial energy=%12.5E, Initial gg=%12.5E\n", utot0, gg0);
    rc = e3d_solve(h, &st);  // :473
  } else {
    if ((rc = e3d_checkpoint_load(h, resume.c_str()))) return fail("e3d_checkpoint_load", rc);
    rc = e3d_iterate(h, max_iter, &st);
  }
  if (rc && rc != E3D_ERR_MAXITER) return fail("e3d_solve", rc);
  if (!ckpt.empty()) {
    const int rs = e3d_checkpoint_save(h, ckpt.c_str());
    if (rs) return fail("e3d_checkpoint_save", rs);
  }
  // per-iteration history (cgitr file, :2019-2021)
  {
    std::vector<double> hist((size_t)std::max(st.iterations, 1));
    int32_t cnt = 0;
    e3d_get_history(h, hist.data(), (int32_t)hist.size(), &cnt);
    const std::string hp = outdir + "/cgitr_SS316L_polycrystal.txt";
    FILE* f = std::fopen(hp.c_str(), "w");
    if (f) {
      for (int i = 0; i < cnt; ++i) std::fprintf(f, "%8d    %20.8E\n", i + 1, hist[(size_t)i]);
      std::fclose(f);
    }
  }
  double utot = 0.0, gg = 0.0;
  if ((rc = e3d_energy(h, &utot, &gg))) return fail("e3d_energy", rc);  // :479
  double strav[6], epsav[6];
  if ((rc = e3d_stress(h, strav, epsav))) return fail("e3d_stress", rc);  // :514
  std::fprintf(out, " Energy= %.10e gg= %.10e\n Number of conjugate steps= %d\n", utot, st.gg, st.iterations);
  std::printf("Energy=%12.5E, gg=%12.5E, rel. residual norm=%12.5E\n Number of conjugate steps= %d\n", utot,
              st.gg, st.rel_res, st.iterations);
  {
    const std::string hp = outdir + "/cg_history_polycrystal.txt";
    FILE* f = std::fopen(hp.c_str(), "w");
    if (f) {
      std::fprintf(f, "%8d %18.10E %18.10E\n", 0, utot0, 1.0);
      std::fprintf(f, "%8d %18.10E %18.10E\n", st.iterations, utot, st.rel_res);
      std::fclose(f);
    }
  }
  std::fprintf(out, " stresses: xx, yy, zz, xz, yz, xy\n");
  for (int k = 0; k < 6; ++k) std::fprintf(out, "%15.6E", strav[k]);
  std::fprintf(out, "\n strains: xx, yy, zz, xz, yz, xy\n");
  for (int k = 0; k < 6; ++k) std::fprintf(out, "%15.6E", epsav[k]);
  std::fprintf(out, "\n");
  const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  std::fprintf(out, "\n Calculation complete!\n Total calculation time: %f seconds\n", elapsed);
  std::printf(" End of CG\n\n Calculation complete!\n Total calculation time: %f seconds\n", elapsed);
  if (json) {  // one metrics line per solve (non-finite values as null)
    auto num = [](double v) {
      char b[40];
      if (std::isfinite(v))
        std::snprintf(b, sizeof b, "%.17g", v);
      else
        std::snprintf(b, sizeof b, "null");
      return std::string(b);
    };
    std::string line = "{\"grid\": [" + std::to_string(nx) + ", " + std::to_string(ny) + ", " + std::to_string(nz) +
                       "], \"dof\": " + std::to_string(3 * ns) + ", \"precision\": \"" +
                       (precision == E3D_PREC_MIXED ? "mixed" : "fp64") + "\", \"criterion\": \"" +
                       (criterion == E3D_CRIT_PRECOND_REL ? "precond" : "ref") + "\", \"iterations\": " +
                       std::to_string(st.iterations) + ", \"exit_reason\": " + std::to_string(st.exit_reason) +
                       ", \"refinements\": " + std::to_string(st.refinements) + ", \"resets\": " +
                       std::to_string(st.resets) + ", \"utot0\": " + num(utot0) + ", \"utot\": " + num(utot) +
                       ", \"rel_res\": " + num(st.rel_res) + ", \"true_rel\": " + num(st.true_rel) +
                       ", \"ms_setup\": " + num(st.ms_setup) + ", \"ms_pcg\": " + num(st.ms_iter) +
                       ", \"seconds_total\": " + num(elapsed) + ", \"dof_iters_per_s\": " +
                       num(st.ms_iter > 0 ? 3.0 * (double)ns * st.iterations / (st.ms_iter * 1e-3) : 0.0);
    line += ", \"strav\": [";
    for (int k = 0; k < 6; ++k) line += num(strav[k]) + (k < 5 ? ", " : "]");
    line += ", \"epsav\": [";
    for (int k = 0; k < 6; ++k) line += num(epsav[k]) + (k < 5 ? ", " : "]");
    line += "}";
    std::printf("%s\n", line.c_str());
    std::fflush(stdout);
  }
  std::fclose(out);
  if (fullfield) {  // stress_fullfield_OpenMP (:2639-2877)
    std::vector<double> sig(6 * (size_t)ns), vm((size_t)ns);
    if ((rc = e3d_stress_field(h, sig.data(), vm.data()))) return fail("e3d_stress_field", rc);
    const std::string fp = outdir + "/fullfield_poly.h5";
    if (e3d_h5_fullfield_write(fp.c_str(), (int64_t)ns, pix.data(), vm.data(), sig.data()) != 0) {
      std::fprintf(stderr, "e3d_run: %s\n", e3d_last_cuda_error());
      e3d_destroy(h);
      return 1;
    }
  }
  e3d_destroy(h);
  return (st.exit_reason == E3D_EXIT_CONVERGED || st.exit_reason == E3D_EXIT_HAH_GUARD) ? 0 : 3;
}
