// A driver in the shape of microLC's simulating_lcurves/src/driver.cpp:19-275, written
// only against the reference's own class and function names and compiled against
// include/microlc_compat.hpp (the JSON input is replaced by fixed values and argv).
//
//   driver_compat <map id A> <map id B> <out dir>
//
// Map ids are directories under MAP_PATH (a compile-time string, as in the reference)
// holding mapmeta.dat and map.bin.  Writes the same outputs as the reference's driver
// (mpd_A/B/R.dat, binned_exp.dat, binned_N.dat, lcurvesA/B.dat) plus likelihood.dat.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "microlc_compat.hpp"

int main(int argc, char* argv[]) {
  if (argc != 4) {
    std::printf("usage: %s map_A map_B out_dir\n", argv[0]);
    return 1;
  }
  const std::string out = std::string(argv[3]) + "/";
  std::vector<double> sizes{0.0, 0.05, 0.1, 0.2, 0.3};
  const int Nprof = (int)sizes.size();
  const std::string shape = "gaussian";

  const double dum_rein = 1.0;
  MagnificationMap mapA(argv[1], dum_rein);
  MagnificationMap mapB(argv[2], dum_rein);

  // grid locations (driver.cpp:50-59)
  const int Nside = 24, Nmap = mapA.Nx;
  const double ss = mapA.width;
  const int Nloc = Nside * Nside;
  std::vector<int> x(Nloc), y(Nloc);
  const int Noff = (int)std::ceil((Nmap / ss) * sizes.back());
  locations_on_grid(Nside, Nmap, Noff, x.data(), y.data());

  SimLC LCA(Nloc, Nprof);
  SimLC LCB(Nloc, Nprof);
  Chi2 chi2(Nloc);

  const int Nd = 5;
  double d[Nd] = {0.7, 1.2, 1.4, 1.1, 0.9};
  double s[Nd] = {0.1, 0.15, 0.1, 0.1, 0.15};
  double t[Nd] = {5.0, 7.0, 12.0, 14.0, 17.0};
  const double DL = 1750, DS = 850, DLS = 1570;
  const double Dfac = std::sqrt(DS * DLS / DL);
  std::printf("Total GPU memory: %ld (MiB)\n", (long)get_total_gpu_mem());

  const int Nbins_mpd = 200, Nbins_ratio = 60;
  const double min_mpd = 0.02, max_mpd = 200, min_ratio = 0.05, max_ratio = 20;
  Chi2SortBins sort_struct(Nloc, Nbins_ratio);

  expanding_source(&mapA, sizes, shape, Nloc, x.data(), y.data(), &LCA);
  expanding_source(&mapB, sizes, shape, Nloc, x.data(), y.data(), &LCB);
  LCA.transfer_to_CPU();
  LCB.transfer_to_CPU();

  Mpd binned_mpd_A = mapA.getBinnedMpd(Nbins_mpd, min_mpd, max_mpd);
  Mpd binned_mpd_B = mapB.getBinnedMpd(Nbins_mpd, min_mpd, max_mpd);
  binned_mpd_A.normalize();
  binned_mpd_B.normalize();
  Mpd ratio(Nbins_ratio, min_ratio, max_ratio, "log");
  binned_mpd_A.divide_by(&binned_mpd_B, &ratio);
  binned_mpd_A.writeMpd(out + "mpd_A.dat");
  binned_mpd_B.writeMpd(out + "mpd_B.dat");
  ratio.writeMpd(out + "mpd_R.dat");

  setup_integral_GPU(&LCA, &LCB, &ratio, &sort_struct);

  std::vector<double> M{0.4, 0.5};
  std::vector<double> V{1};
  std::vector<double> binned_chi2(Nbins_ratio), binned_exp(Nbins_ratio);
  Chi2Vars chi2_vars = setup_chi2_calculation(M, V, Dfac, Nd, d, t, s, Nprof, sizes.data());
  calculate_chi2_GPU(&chi2_vars, chi2.d_values, &sort_struct, &LCA, &LCB);
  bin_chi2_GPU(binned_chi2.data(), binned_exp.data(), &sort_struct, chi2.d_values);
  const double integral = trapezium(ratio.Nbins, binned_exp.data(), ratio.counts, ratio.bins);
  const double like = integral * std::exp(-0.5 * chi2_vars.const_term);

  FILE* fh = std::fopen((out + "binned_exp.dat").c_str(), "w");
  FILE* fh2 = std::fopen((out + "binned_N.dat").c_str(), "w");
  for (int i = 0; i < sort_struct.Nbins; i++) {
    std::fprintf(fh, "%.17g %.17g %.17g\n", ratio.bins[i], binned_exp[i], binned_chi2[i]);
    std::fprintf(fh2, "%.17g %d\n", ratio.bins[i], sort_struct.n_per_bin[i]);
  }
  std::fclose(fh);
  std::fclose(fh2);
  fh = std::fopen((out + "lcurvesA.dat").c_str(), "w");
  fh2 = std::fopen((out + "lcurvesB.dat").c_str(), "w");
  for (int i = 0; i < Nloc; i++) {
    for (int j = 0; j < Nprof; j++) {
      std::fprintf(fh, " %.17g", LCA.LC[i * Nprof + j]);
      std::fprintf(fh2, " %.17g", LCB.LC[i * Nprof + j]);
    }
    std::fprintf(fh, "\n");
    std::fprintf(fh2, "\n");
  }
  std::fclose(fh);
  std::fclose(fh2);
  fh = std::fopen((out + "likelihood.dat").c_str(), "w");
  std::fprintf(fh, "%.17g %.17g %d %.17g\n", like, integral, chi2_vars.Njp, chi2_vars.const_term);
  std::fclose(fh);
  // full-precision MPDs for the parity check (writeMpd keeps 7 digits, like the reference)
  fh = std::fopen((out + "mpd_full.dat").c_str(), "w");
  for (int i = 0; i < Nbins_mpd; i++)
    std::fprintf(fh, "%.17g %.17g %.17g %.17g\n", binned_mpd_A.bins[i], binned_mpd_A.counts[i], binned_mpd_B.bins[i],
                 binned_mpd_B.counts[i]);
  for (int i = 0; i < Nbins_ratio; i++) std::fprintf(fh, "%.17g %.17g 0 0\n", ratio.bins[i], ratio.counts[i]);
  std::fclose(fh);
  std::printf("likelihood %.17g\n", like);
  return 0;
}
