// microlc -- the light-curve simulator's command-line driver (simulating_lcurves/src/
// driver.cpp:19-275) on this library.  Same JSON input, same output files, same last line
// "GPU: <integral>" (the line repeat.sh:27 scrapes).
//
//   microlc input.json [--out DIR] [--check] [--full-precision]
//
// Input keys kept from the reference (driver.cpp:41-120):
//   sizes[]             half-light radii in Einstein radii, sizes[0] = 0 (the point source)
//   shape               uniform | gaussian | thermal_hole | exponential
//   locations           {type: grid, Nmap, ss, Nside} | {type: random, Nmap, ss, Nloc, seed}
//   mpds                {mpd: {Nbins, min, max}, ratio: {Nbins, min, max}}
//   DL, DS, DLS         distances (Mpc)
//   data[0]             {d[], s[], t[]}: observed flux ratios, errors, epochs
// Keys added here (all optional; defaults are the reference's hard-coded values):
//   maps                {path: "<dir prefix>", A: "12123", B: "11156"}  (driver.cpp:133-134;
//                       the prefix defaults to $MLC_MAP_PATH, the compile-time MAP_PATH of
//                       the reference)
//   M, V                [M_A, M_B] and [V] of setup_chi2_calculation (driver.cpp:195-196)
//   locations           {type: tracks, Nmap, ss, Ntracks, seed, v: [vmin, vmax]}: straight
//                       tracks in place of fixed locations (v in Einstein radii per unit of
//                       t); light curves of every profile on both maps at the epochs of
//                       data[0] (map A) and data[1] (map B, else data[0]), and the
//                       offset-minimised chi2 of each against d (magnitudes), s (errors).
// Options: --out DIR writes the files there (default: the working directory); --check
// validates the input and prints the resolved settings as one JSON line without touching
// the GPU; --full-precision writes every number with 17 significant digits (the
// reference's formats keep 6 or 7) and adds likelihood.dat.
//
// Differences from the reference's driver, by design: a missing or mistyped key, a
// malformed file, a size other than 0 first, locations outside the map or maps of
// different sizes stop the run with a message naming the problem (exit status 1) instead
// of reading 0 or out of range; there is no 50-epoch limit (driver.cpp:85-93);
// gaussian_hole and wavy are refused because the reference's driver never sets their Rin
// and a (gpu_functions.cu:105-110); lcurvesA/B.dat hold the computed light curves (the
// reference writes its host arrays without copying them back from the GPU).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "json.hpp"
#include "microlc_compat.hpp"

namespace {

using mlcjson::Value;

struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

std::string join(const std::string& a, const std::string& b) { return a.empty() ? b : a + "." + b; }

const Value& member(const Value& obj, const std::string& key, const std::string& where, bool required = true) {
  if (obj.type != Value::Object) throw InputError((where.empty() ? "input" : where) + ": expected an object");
  if (required && !obj.has(key)) throw InputError(join(where, key) + ": missing");
  return obj[key];
}

double number(const Value& v, const std::string& path) {
  if (v.type != Value::Number)
    throw InputError(path + ": expected a number, found " + Value::type_name(v.type));
  return v.num;
}

int integer(const Value& v, const std::string& path) {
  const double x = number(v, path);
  if (x != std::floor(x) || x < -2147483648.0 || x > 2147483647.0)
    throw InputError(path + ": expected an integer, found " + std::to_string(x));
  return (int)x;
}

std::string text(const Value& v, const std::string& path) {
  if (v.type != Value::String)
    throw InputError(path + ": expected a string, found " + Value::type_name(v.type));
  return v.str;
}

std::vector<double> numbers(const Value& v, const std::string& path, size_t min_len) {
  if (v.type != Value::Array) throw InputError(path + ": expected an array, found " + Value::type_name(v.type));
  if (v.size() < min_len) throw InputError(path + ": needs at least " + std::to_string(min_len) + " entries");
  std::vector<double> out(v.size());
  for (size_t i = 0; i < v.size(); i++) out[i] = number(v[i], path + "[" + std::to_string(i) + "]");
  return out;
}

void positive(double x, const std::string& path) {
  if (!(x > 0)) throw InputError(path + ": must be positive");
}

struct Bins {
  int Nbins = 0;
  double min = 0, max = 0;
};

struct Series {
  std::vector<double> d, s, t;
};

struct Config {
  std::vector<double> sizes;
  std::string shape;
  std::string loc_type;
  int Nmap = 0, Nside = 0, Nloc = 0, seed = 0, Noff = 0;
  double ss = 0;
  int Ntracks = 0;
  double vmin = 0, vmax = 0;
  Bins mpd, ratio;
  double DL = 0, DS = 0, DLS = 0, Dfac = 0;
  std::vector<Series> data;
  std::vector<double> M{0.4, 0.5}, V{1.0};
  std::string map_path, idA{"12123"}, idB{"11156"};
};

Bins read_bins(const Value& v, const std::string& where) {
  Bins b;
  b.Nbins = integer(member(v, "Nbins", where), where + ".Nbins");
  b.min = number(member(v, "min", where), where + ".min");
  b.max = number(member(v, "max", where), where + ".max");
  if (b.Nbins < 1) throw InputError(where + ".Nbins: must be at least 1");
  if (!(b.min > 0) || !(b.max > b.min)) throw InputError(where + ": needs 0 < min < max (log-spaced bins)");
  return b;
}

Series read_series(const Value& v, const std::string& where) {
  Series s;
  s.d = numbers(member(v, "d", where), where + ".d", 1);
  s.s = numbers(member(v, "s", where), where + ".s", 1);
  s.t = numbers(member(v, "t", where), where + ".t", 1);
  if (s.s.size() != s.d.size() || s.t.size() != s.d.size())
    throw InputError(where + ": d, s and t must have the same length");
  for (size_t i = 0; i < s.s.size(); i++) positive(s.s[i], where + ".s[" + std::to_string(i) + "]");
  return s;
}

Config read_config(const Value& in) {
  Config c;
  if (in.type != Value::Object) throw InputError("input: expected a JSON object at the top level");
  c.sizes = numbers(member(in, "sizes", ""), "sizes", 1);
  if (c.sizes[0] != 0.0) throw InputError("sizes[0]: must be 0 (the point source comes first)");
  for (size_t i = 1; i < c.sizes.size(); i++)
    if (!(c.sizes[i] > 0)) throw InputError("sizes[" + std::to_string(i) + "]: must be positive");
  c.shape = text(member(in, "shape", ""), "shape");
  if (c.shape == "gaussian_hole" || c.shape == "wavy")
    throw InputError("shape: '" + c.shape + "' needs profile parameters (Rin, a) that this input format has no keys for");
  if (c.shape != "uniform" && c.shape != "gaussian" && c.shape != "thermal_hole" && c.shape != "exponential")
    throw InputError("shape: unknown profile shape '" + c.shape + "'");

  const Value& loc = member(in, "locations", "");
  c.loc_type = text(member(loc, "type", "locations"), "locations.type");
  c.Nmap = integer(member(loc, "Nmap", "locations"), "locations.Nmap");
  c.ss = number(member(loc, "ss", "locations"), "locations.ss");
  if (c.Nmap < 2) throw InputError("locations.Nmap: must be at least 2");
  positive(c.ss, "locations.ss");
  c.Noff = (int)std::ceil((c.Nmap / c.ss) * c.sizes.back());  // driver.cpp:60, 68
  if (2 * c.Noff >= c.Nmap) throw InputError("locations: the largest profile leaves no room on a map of Nmap pixels");
  if (c.loc_type == "grid") {
    c.Nside = integer(member(loc, "Nside", "locations"), "locations.Nside");
    if (c.Nside < 1) throw InputError("locations.Nside: must be at least 1");
    if ((long long)c.Nside * c.Nside > 46340LL * 46340LL) throw InputError("locations.Nside: too many locations");
    c.Nloc = c.Nside * c.Nside;
  } else if (c.loc_type == "random") {
    c.Nloc = integer(member(loc, "Nloc", "locations"), "locations.Nloc");
    c.seed = integer(member(loc, "seed", "locations"), "locations.seed");
    if (c.Nloc < 1 || c.Nloc > 46340) throw InputError("locations.Nloc: must be in 1..46340");
  } else if (c.loc_type == "tracks") {
    c.Ntracks = integer(member(loc, "Ntracks", "locations"), "locations.Ntracks");
    c.seed = integer(member(loc, "seed", "locations"), "locations.seed");
    const std::vector<double> v = numbers(member(loc, "v", "locations"), "locations.v", 2);
    if (v.size() != 2) throw InputError("locations.v: expected [vmin, vmax]");
    c.vmin = v[0];
    c.vmax = v[1];
    if (!(c.vmin >= 0) || !(c.vmax >= c.vmin)) throw InputError("locations.v: needs 0 <= vmin <= vmax");
    if (c.Ntracks < 1) throw InputError("locations.Ntracks: must be at least 1");
  } else {
    throw InputError("locations.type: expected \"grid\", \"random\" or \"tracks\", found \"" + c.loc_type + "\"");
  }

  const Value& mp = member(in, "mpds", "", c.loc_type != "tracks");
  if (!mp.is_null()) {
    c.mpd = read_bins(member(mp, "mpd", "mpds"), "mpds.mpd");
    c.ratio = read_bins(member(mp, "ratio", "mpds"), "mpds.ratio");
  }
  c.DL = number(member(in, "DL", "", c.loc_type != "tracks"), "DL");
  c.DS = number(member(in, "DS", "", c.loc_type != "tracks"), "DS");
  c.DLS = number(member(in, "DLS", "", c.loc_type != "tracks"), "DLS");
  if (c.loc_type != "tracks") {
    positive(c.DL, "DL");
    positive(c.DS, "DS");
    positive(c.DLS, "DLS");
    c.Dfac = std::sqrt(c.DS * c.DLS / c.DL);  // driver.cpp:105
  }
  const Value& data = member(in, "data", "");
  if (data.type != Value::Array || data.size() < 1) throw InputError("data: expected an array of at least one entry");
  for (size_t i = 0; i < data.size() && i < 2; i++) c.data.push_back(read_series(data[i], "data[" + std::to_string(i) + "]"));
  if (c.loc_type != "tracks") c.data.resize(1);

  if (in.has("M")) c.M = numbers(in["M"], "M", 2);
  if (in.has("V")) c.V = numbers(in["V"], "V", 1);
  for (size_t i = 0; i < c.M.size(); i++) positive(c.M[i], "M[" + std::to_string(i) + "]");
  for (size_t i = 0; i < c.V.size(); i++) positive(c.V[i], "V[" + std::to_string(i) + "]");
  if (const char* e = std::getenv("MLC_MAP_PATH")) c.map_path = e;
  if (in.has("maps")) {
    const Value& m = in["maps"];
    if (m.type != Value::Object) throw InputError("maps: expected an object");
    if (m.has("path")) c.map_path = text(m["path"], "maps.path");
    if (m.has("A")) c.idA = text(m["A"], "maps.A");
    if (m.has("B")) c.idB = text(m["B"], "maps.B");
  }
  return c;
}

struct Tracks {
  std::vector<double> x0, y0, phi, v;
};

// Straight tracks drawn with std::mt19937_64 (its output sequence is fixed by the C++
// standard, so the tracks are the same on every platform): direction uniform in [0, 2 pi),
// speed uniform in [vmin, vmax] (Einstein radii per unit of t, converted to pixels), the
// midpoint uniform in the square that keeps the whole track, over the epochs [tmin, tmax],
// at least Noff + 1 pixels from every edge.
Tracks make_tracks(const Config& c, double tmin, double tmax) {
  std::mt19937_64 gen((uint64_t)(uint32_t)c.seed);
  auto uni = [&](double a, double b) { return a + (b - a) * ((double)(gen() >> 11) * 0x1.0p-53); };
  const double pix_per_re = c.Nmap / c.ss;
  const double tmid = 0.5 * (tmin + tmax);
  Tracks tr;
  for (int i = 0; i < c.Ntracks; i++) {
    const double phi = uni(0.0, 2.0 * M_PI);
    const double v = uni(c.vmin, c.vmax) * pix_per_re;
    const double half = 0.5 * v * (tmax - tmin);
    const double lo = c.Noff + 1.0 + half, hi = c.Nmap - c.Noff - 1.0 - half;
    if (!(hi > lo))
      throw InputError("locations.v: a track of speed " + std::to_string(v / pix_per_re) +
                       " over the epochs of data does not fit in the map");
    const double xm = uni(lo, hi), ym = uni(lo, hi);
    tr.x0.push_back(xm - v * tmid * std::cos(phi));
    tr.y0.push_back(ym - v * tmid * std::sin(phi));
    tr.phi.push_back(phi);
    tr.v.push_back(v);
  }
  return tr;
}

std::string fmt(double x) {
  char b[40];
  std::snprintf(b, sizeof b, "%.17g", x);
  return b;
}

void print_check(const Config& c) {
  std::ostringstream o;
  o << "{\"Nprof\": " << c.sizes.size() << ", \"shape\": \"" << c.shape << "\", \"locations\": \"" << c.loc_type
    << "\", \"Nmap\": " << c.Nmap << ", \"Noff\": " << c.Noff;
  if (c.loc_type == "tracks") {
    const std::vector<double>& t = c.data[0].t;
    const Tracks tr = make_tracks(c, *std::min_element(t.begin(), t.end()), *std::max_element(t.begin(), t.end()));
    double sx = 0, sy = 0, sp = 0, sv = 0;
    for (int i = 0; i < c.Ntracks; i++) {
      sx += tr.x0[i];
      sy += tr.y0[i];
      sp += tr.phi[i];
      sv += tr.v[i];
    }
    o << ", \"Ntracks\": " << c.Ntracks << ", \"track_sums\": [" << fmt(sx) << ", " << fmt(sy) << ", " << fmt(sp)
      << ", " << fmt(sv) << "]";
  } else {
    std::vector<int> x(c.Nloc), y(c.Nloc);
    if (c.loc_type == "grid")
      microlc_compat::check_status(mlc_locations_grid(c.Nside, c.Nmap, c.Noff, x.data(), y.data()), "locations");
    else
      microlc_compat::check_status(mlc_locations_random(c.Nloc, c.Nmap, c.Noff, c.seed, x.data(), y.data()),
                                   "locations");
    long long sx = 0, sy = 0;
    for (int i = 0; i < c.Nloc; i++) {
      sx += x[i];
      sy += y[i];
    }
    o << ", \"Nloc\": " << c.Nloc << ", \"x_sum\": " << sx << ", \"y_sum\": " << sy << ", \"Dfac\": " << fmt(c.Dfac)
      << ", \"mpd\": [" << c.mpd.Nbins << ", " << fmt(c.mpd.min) << ", " << fmt(c.mpd.max) << "], \"ratio\": ["
      << c.ratio.Nbins << ", " << fmt(c.ratio.min) << ", " << fmt(c.ratio.max) << "]";
  }
  o << ", \"Nd\": " << c.data[0].d.size() << ", \"M\": [";
  for (size_t i = 0; i < c.M.size(); i++) o << (i ? ", " : "") << fmt(c.M[i]);
  o << "], \"V\": [";
  for (size_t i = 0; i < c.V.size(); i++) o << (i ? ", " : "") << fmt(c.V[i]);
  o << "], \"maps\": [\"" << c.map_path + c.idA << "\", \"" << c.map_path + c.idB << "\"]}";
  std::printf("%s\n", o.str().c_str());
}

FILE* open_out(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) throw std::runtime_error("cannot write " + path);
  return f;
}

void check_map(const MagnificationMap& m, const Config& c, const std::string& name) {
  if (m.Nx < c.Nmap)
    throw InputError("locations.Nmap: " + std::to_string(c.Nmap) + " is larger than map " + name + " (" +
                     std::to_string(m.Nx) + " pixels)");
}

// The reference's flow (driver.cpp:128-266): light curves at fixed locations on both
// maps, map MPDs and their ratio, pair ranks, ratio chi2, binning, the trapezium integral.
int run_locations(const Config& c, const std::string& out, bool full) {
  const int Nprof = (int)c.sizes.size();
  std::printf("Number of profiles set to: %d (%s)\n", Nprof, c.shape.c_str());
  std::vector<int> x(c.Nloc), y(c.Nloc);
  if (c.loc_type == "grid")
    microlc_compat::check_status(mlc_locations_grid(c.Nside, c.Nmap, c.Noff, x.data(), y.data()), "locations");
  else
    microlc_compat::check_status(mlc_locations_random(c.Nloc, c.Nmap, c.Noff, c.seed, x.data(), y.data()),
                                 "locations");
  std::printf("Sampling from %d locations per map (%s).\n", c.Nloc, c.loc_type.c_str());
  const int Nd = (int)c.data[0].d.size();
  std::printf("Data length: %d\n", Nd);
  std::printf("Total GPU memory: %ld (bytes)\n", (long)get_total_gpu_mem());

  SimLC LCA(c.Nloc, Nprof);
  SimLC LCB(c.Nloc, Nprof);
  Chi2 chi2(c.Nloc);
  Chi2SortBins sort_struct(c.Nloc, c.ratio.Nbins);

  const double dum_rein = 1.0;
  MagnificationMap mapA(c.map_path + c.idA, dum_rein);
  MagnificationMap mapB(c.map_path + c.idB, dum_rein);
  check_map(mapA, c, "A");
  check_map(mapB, c, "B");
  if (mapA.Nx != mapB.Nx) throw InputError("maps: A and B must have the same size");

  std::cout << "CONVOLUTIONS" << std::endl << std::string(100, '*') << std::endl;
  expanding_source(&mapA, c.sizes, c.shape, c.Nloc, x.data(), y.data(), &LCA);
  expanding_source(&mapB, c.sizes, c.shape, c.Nloc, x.data(), y.data(), &LCB);
  LCA.transfer_to_CPU();
  LCB.transfer_to_CPU();

  std::cout << "MPDS" << std::endl << std::string(100, '*') << std::endl;
  Mpd mpdA = mapA.getBinnedMpd(c.mpd.Nbins, c.mpd.min, c.mpd.max);
  Mpd mpdB = mapB.getBinnedMpd(c.mpd.Nbins, c.mpd.min, c.mpd.max);
  mpdA.normalize();
  mpdB.normalize();
  Mpd ratio(c.ratio.Nbins, c.ratio.min, c.ratio.max, "log");
  mpdA.divide_by(&mpdB, &ratio);
  const char* f2 = full ? "%.17g %.17g\n" : "%11.6e %11.6e\n";
  for (const auto& [name, m] : {std::pair<const char*, Mpd*>{"mpd_A.dat", &mpdA}, {"mpd_B.dat", &mpdB},
                                {"mpd_R.dat", &ratio}}) {
    FILE* f = open_out(out + name);
    for (int i = 0; i < m->Nbins; i++) std::fprintf(f, f2, m->bins[i], m->counts[i]);
    std::fclose(f);
  }
  setup_integral_GPU(&LCA, &LCB, &ratio, &sort_struct);

  std::cout << "CHI-SQUARED" << std::endl << std::string(100, '*') << std::endl;
  std::vector<double> bchi2(c.ratio.Nbins), bexp(c.ratio.Nbins);
  std::vector<double> d = c.data[0].d, s = c.data[0].s, t = c.data[0].t;
  Chi2Vars cv = setup_chi2_calculation(c.M, c.V, c.Dfac, Nd, d.data(), t.data(), s.data(), Nprof,
                                       const_cast<double*>(c.sizes.data()));
  calculate_chi2_GPU(&cv, chi2.d_values, &sort_struct, &LCA, &LCB);
  bin_chi2_GPU(bchi2.data(), bexp.data(), &sort_struct, chi2.d_values);
  const double integral = trapezium(ratio.Nbins, bexp.data(), ratio.counts, ratio.bins);
  const double like = integral * std::exp(-0.5 * cv.const_term);  // driver.cpp:234

  FILE* fe = open_out(out + "binned_exp.dat");
  FILE* fn = open_out(out + "binned_N.dat");
  for (int i = 0; i < sort_struct.Nbins; i++) {
    if (full)
      std::fprintf(fe, "%.17g %.17g %.17g\n", ratio.bins[i], bexp[i], bchi2[i]);
    else
      std::fprintf(fe, "%11.6e %11.6e\n", ratio.bins[i], bexp[i]);
    std::fprintf(fn, full ? "%.17g %d\n" : "%11.6e %d\n", ratio.bins[i], (int)sort_struct.n_per_bin[i]);
  }
  std::fclose(fe);
  std::fclose(fn);
  FILE* fa = open_out(out + "lcurvesA.dat");
  FILE* fb = open_out(out + "lcurvesB.dat");
  const char* f1 = full ? " %.17g" : " %f";
  for (int i = 0; i < c.Nloc; i++) {
    for (int j = 0; j < Nprof; j++) {
      std::fprintf(fa, f1, LCA.LC[(size_t)i * Nprof + j]);
      std::fprintf(fb, f1, LCB.LC[(size_t)i * Nprof + j]);
    }
    std::fprintf(fa, "\n");
    std::fprintf(fb, "\n");
  }
  std::fclose(fa);
  std::fclose(fb);
  if (full) {
    FILE* fl = open_out(out + "likelihood.dat");
    std::fprintf(fl, "%.17g %.17g %d %.17g\n", like, integral, cv.Njp, cv.const_term);
    std::fclose(fl);
  }
  std::cout << "GPU: " << integral << std::endl;  // driver.cpp:231
  return 0;
}

template <class T>
T* dev_alloc(size_t n) {
  return microlc_compat::device_alloc<T>(n, "microlc: cudaMalloc");
}

void to_dev(void* dst, const void* src, size_t bytes) {
  microlc_compat::check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "microlc: upload");
}

// Light curves of every profile along the tracks on one map at the epochs of one observed
// series, and each curve's offset-minimised chi2 against it.  lc[(q*ntracks + i)*T + e],
// chi2/dm[q*ntracks + i].
void track_curves(mlc_ctx* ctx, MagnificationMap& map, const Config& c, const Tracks& tr, const Series& obs,
                  std::vector<double>& lc, std::vector<double>& chi2, std::vector<double>& dm) {
  const int Nprof = (int)c.sizes.size(), n = c.Ntracks, T = (int)obs.t.size();
  const int64_t E = (int64_t)n * T;
  mlc_map* m = nullptr;
  microlc_compat::check(mlc_map_create(ctx, map.data, 0, MLC_F64, map.Nx, map.Ny, MLC_F64, &m), "mlc_map_create");
  std::vector<int64_t> off(n + 1);
  std::vector<double> t((size_t)E);
  for (int i = 0; i <= n; i++) off[i] = (int64_t)i * T;
  for (int i = 0; i < n; i++)
    for (int e = 0; e < T; e++) t[(size_t)i * T + e] = obs.t[e];
  double *dx0 = dev_alloc<double>(n), *dy0 = dev_alloc<double>(n), *dphi = dev_alloc<double>(n),
         *dv = dev_alloc<double>(n), *dt = dev_alloc<double>(E), *dlc = dev_alloc<double>((size_t)Nprof * E),
         *dchi = dev_alloc<double>((size_t)Nprof * n), *ddm = dev_alloc<double>((size_t)Nprof * n);
  int64_t* doff = dev_alloc<int64_t>(n + 1);
  to_dev(dx0, tr.x0.data(), n * sizeof(double));
  to_dev(dy0, tr.y0.data(), n * sizeof(double));
  to_dev(dphi, tr.phi.data(), n * sizeof(double));
  to_dev(dv, tr.v.data(), n * sizeof(double));
  to_dev(dt, t.data(), E * sizeof(double));
  to_dev(doff, off.data(), (n + 1) * sizeof(int64_t));
  // point source: the map itself
  void* pix = nullptr;
  microlc_compat::check(mlc_map_data(m, &pix), "mlc_map_data");
  const void* maps0[1] = {pix};
  microlc_compat::check(mlc_sample_tracks(ctx, maps0, 1, map.Nx, map.Ny, MLC_F64, n, dx0, dy0, dphi, dv, doff, dt,
                                          /*mag*/ 1, dlc),
                        "mlc_sample_tracks");
  if (Nprof > 1) {
    std::vector<mlc_profile> prof(Nprof - 1);
    for (int k = 1; k < Nprof; k++) {
      mlc_profile& p = prof[k - 1];
      p = mlc_profile{};
      p.shape = microlc_compat::shape_code(c.shape);
      p.ref_compat = 1;
      p.pix = map.pixSizePhys;
      p.rhalf = c.sizes[k] * map.pixSizePhys * map.Nx / map.width;  // gpu_functions.cu:184
    }
    mlc_tracks tk{n, E, dx0, dy0, dphi, dv, doff, dt};
    microlc_compat::check(mlc_convolve_sample_tracks(ctx, m, nullptr, Nprof - 1, prof.data(), &tk, MLC_CONV_FUSED,
                                                     /*mag*/ 1, dlc + E, 0),
                          "mlc_convolve_sample_tracks");
  }
  std::vector<double> w(T);
  for (int e = 0; e < T; e++) w[e] = 1.0 / (obs.s[e] * obs.s[e]);
  microlc_compat::check(mlc_chi2_offset(ctx, MLC_F64, Nprof * n, T, dlc, obs.d.data(), w.data(), dchi, ddm),
                        "mlc_chi2_offset");
  microlc_compat::check(mlc_ctx_synchronize(ctx), "mlc_ctx_synchronize");
  lc.resize((size_t)Nprof * E);
  chi2.resize((size_t)Nprof * n);
  dm.resize((size_t)Nprof * n);
  microlc_compat::check_cuda(cudaMemcpy(lc.data(), dlc, lc.size() * sizeof(double), cudaMemcpyDeviceToHost), "lc");
  microlc_compat::check_cuda(cudaMemcpy(chi2.data(), dchi, chi2.size() * sizeof(double), cudaMemcpyDeviceToHost),
                             "chi2");
  microlc_compat::check_cuda(cudaMemcpy(dm.data(), ddm, dm.size() * sizeof(double), cudaMemcpyDeviceToHost), "dm");
  for (void* p : {(void*)dx0, (void*)dy0, (void*)dphi, (void*)dv, (void*)dt, (void*)dlc, (void*)dchi, (void*)ddm,
                  (void*)doff})
    cudaFree(p);
  mlc_map_destroy(m);
}

int run_tracks(const Config& c, const std::string& out, bool full) {
  const int Nprof = (int)c.sizes.size(), n = c.Ntracks;
  std::printf("Number of profiles set to: %d (%s)\n", Nprof, c.shape.c_str());
  const Series& sA = c.data[0];
  const Series& sB = c.data.size() > 1 ? c.data[1] : c.data[0];
  double tmin = sA.t[0], tmax = sA.t[0];
  for (const Series* s : {&sA, &sB})
    for (double x : s->t) {
      tmin = std::min(tmin, x);
      tmax = std::max(tmax, x);
    }
  const Tracks tr = make_tracks(c, tmin, tmax);
  std::printf("Sampling %d tracks per map at %zu and %zu epochs.\n", n, sA.t.size(), sB.t.size());
  const double dum_rein = 1.0;
  MagnificationMap mapA(c.map_path + c.idA, dum_rein);
  MagnificationMap mapB(c.map_path + c.idB, dum_rein);
  check_map(mapA, c, "A");
  check_map(mapB, c, "B");
  mlc_ctx* ctx = microlc_compat::context();

  FILE* ft = open_out(out + "tracks.dat");
  for (int i = 0; i < n; i++) std::fprintf(ft, "%.17g %.17g %.17g %.17g\n", tr.x0[i], tr.y0[i], tr.phi[i], tr.v[i]);
  std::fclose(ft);
  double best = INFINITY;
  int best_i = -1, best_q = -1;
  char best_map = 'A';
  for (int which = 0; which < 2; which++) {
    MagnificationMap& map = which ? mapB : mapA;
    const Series& s = which ? sB : sA;
    const char tag = which ? 'B' : 'A';
    std::vector<double> lc, chi2, dm;
    track_curves(ctx, map, c, tr, s, lc, chi2, dm);
    const int T = (int)s.t.size();
    const int64_t E = (int64_t)n * T;
    FILE* fl = open_out(out + "lcurves_tracks_" + tag + ".dat");
    FILE* fc = open_out(out + "chi2_tracks_" + tag + ".dat");
    const char* f1 = full ? " %.17g" : " %f";
    for (int i = 0; i < n; i++) {
      for (int q = 0; q < Nprof; q++)
        for (int e = 0; e < T; e++) std::fprintf(fl, f1, lc[(size_t)q * E + (size_t)i * T + e]);
      std::fprintf(fl, "\n");
      for (int q = 0; q < Nprof; q++) {
        const double x = chi2[(size_t)q * n + i];
        std::fprintf(fc, full ? " %.17g %.17g" : " %11.6e %11.6e", x, dm[(size_t)q * n + i]);
        if (x < best) {
          best = x;
          best_i = i;
          best_q = q;
          best_map = tag;
        }
      }
      std::fprintf(fc, "\n");
    }
    std::fclose(fl);
    std::fclose(fc);
  }
  std::cout << "best chi2: " << best << " (map " << best_map << ", track " << best_i << ", size " << best_q << ")"
            << std::endl;
  return 0;
}

std::string read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw InputError("cannot open " + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

}  // namespace

int main(int argc, char* argv[]) {
  std::string input, out;
  bool check = false, full = false;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    if (a == "--check") {
      check = true;
    } else if (a == "--full-precision") {
      full = true;
    } else if (a == "--out" && i + 1 < argc) {
      out = argv[++i];
    } else if (!a.empty() && a[0] != '-' && input.empty()) {
      input = a;
    } else {
      input.clear();
      break;
    }
  }
  if (input.empty()) {
    std::cout << "Error: You need to provide the name of a .json file that contains all the input variables!"
              << std::endl;
    std::cout << "usage: microlc input.json [--out DIR] [--check] [--full-precision]" << std::endl;
    return 1;
  }
  if (!out.empty() && out.back() != '/') out += '/';
  Config c;
  try {
    mlcjson::Value v;
    try {
      v = mlcjson::parse(read_file(input));
    } catch (const mlcjson::ParseError& e) {
      throw InputError(input + ": " + e.what());
    }
    c = read_config(v);
    if (check) {
      print_check(c);
      return 0;
    }
  } catch (const InputError& e) {
    std::cerr << "microlc: " << e.what() << std::endl;
    return 1;
  } catch (const std::exception& e) {
    std::cerr << "microlc: " << e.what() << std::endl;
    return 1;
  }
  try {
    return c.loc_type == "tracks" ? run_tracks(c, out, full) : run_locations(c, out, full);
  } catch (const InputError& e) {
    std::cerr << "microlc: " << e.what() << std::endl;
    return 1;
  } catch (const std::exception& e) {
    std::cerr << "microlc: " << e.what() << std::endl;
    return 2;
  }
}
