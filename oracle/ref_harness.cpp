// Harness driver for the UNMODIFIED HAIL-CAESAR sources (test infrastructure).
//
// Built by oracle/Makefile from the reference's own source files, where they
// lie, into oracle/_ref/ref_harness.  It is the pin for the CPU restatement in
// oracle/hc_oracle.cpp: both are run on the same synthetic inputs and their
// in-memory FP64 state is compared (the reference's .asc writer keeps only 6
// significant digits, LSDRaster.cpp:1216, so files cannot carry the
// comparison).
//
// The call sequence is the one of src/main.cpp:139-204 with three harness
// changes, all optional and applied identically to the restatement:
//   * an iteration limit (main.cpp loops until cycle/60 >= maxcycle);
//   * `lateral`  : calls call_lateral() after call_erosion(), the line that
//                  main.cpp:178 leaves commented out;
//   * `nohill`   : skips slope_creep() and call_global_landsliding()
//                  (main.cpp:186-187), which sit outside the per-step path.
// Output writers (write_output_timeseries, save_raster_output) are not called.
//
// Private members are reached by compiling this one translation unit with
// `private` defined as `public` before the model header; the reference
// translation units are compiled unchanged.

#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <sys/stat.h>
#include <chrono>
#include <omp.h>

#define private public
#include "catchmentmodel/LSDCatchmentModel.hpp"
#undef private
#include "catchmentmodel/LSDRainfallRunoff.hpp"

namespace {

struct Dump {
  FILE* f;
  void put(const char* name, char code, const void* data, uint64_t count,
           size_t elsize) {
    char nm[32] = {0};
    std::strncpy(nm, name, 31);
    fwrite(nm, 1, 32, f);
    fwrite(&code, 1, 1, f);
    fwrite(&count, 8, 1, f);
    fwrite(data, elsize, count, f);
  }
  template <class T>
  void arr2(const char* name, char code, TNT::Array2D<T>& a) {
    if (a.dim1() <= 0 || a.dim2() <= 0) return;
    put(name, code, &a[0][0], (uint64_t)a.dim1() * a.dim2(), sizeof(T));
  }
  template <class T>
  void arr3(const char* name, char code, TNT::Array3D<T>& a) {
    if (a.dim1() <= 0 || a.dim2() <= 0 || a.dim3() <= 0) return;
    put(name, code, &a[0][0][0],
        (uint64_t)a.dim1() * a.dim2() * a.dim3(), sizeof(T));
  }
  void dbl(const char* name, double v) { put(name, 'd', &v, 1, 8); }
};

void read_overrides(const std::string& fn, LSDCatchmentModel& s) {
  std::ifstream in(fn);
  std::string key;
  while (in >> key) {
    if (key == "d") {
      in >> s.d1 >> s.d2 >> s.d3 >> s.d4 >> s.d5 >> s.d6 >> s.d7 >> s.d8 >> s.d9;
    } else if (key == "dprop") {
      for (int n = 0; n < 11; n++) in >> s.dprop[n];
    } else if (key == "fallvel") {
      for (int n = 0; n < 10; n++) in >> s.fallVelocity[n];
    } else {
      std::cerr << "unknown override key " << key << std::endl;
      std::exit(2);
    }
  }
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc < 5) {
    std::cerr << "usage: ref_harness <path/> <file.params> <iters> <out.bin> "
                 "[overrides] [lateral] [nohill]\n";
    return 2;
  }
  std::string pname(argv[1]), pfname(argv[2]);
  long iters = std::atol(argv[3]);
  std::string outfn(argv[4]);
  std::string overrides;
  bool lateral = false, nohill = false;
  for (int a = 5; a < argc; a++) {
    std::string s(argv[a]);
    if (s == "lateral") lateral = true;
    else if (s == "nohill") nohill = true;
    else overrides = s;
  }

  LSDCatchmentModel sim(pname, pfname);
  sim.initialise_model_domain_extents();
  sim.initialise_arrays();
  sim.load_data();
  if (!overrides.empty()) read_overrides(overrides, sim);
  sim.set_time_counters();
  runoffGrid runoff(sim.get_imax(), sim.get_jmax());
  sim.initialise_rainfall_runoff(runoff);
  sim.initialise_drainage_area();

  const int in_channel_landslide_iter_interval = 10;
  const int creep_time_interval_days = 14400;
  const int scan_area_interval_iter = 5;
  const int global_landsliding_interval_hours = 1440;
  const int vegetation_growth_interval_hours = 1440;
  const double creep_coeff = 0.028;

  FILE* steps = std::fopen((outfn + ".steps").c_str(), "wb");
  long it = 0;
  auto t0 = std::chrono::steady_clock::now();
  do {
    sim.set_loop_cycle();
    sim.set_inputoutput_diff();
    sim.set_maximum_timestep();
    sim.increment_counters();
    sim.reach_water_and_sediment_input();
    sim.catchment_waterinputs(runoff);
    sim.flow_route();
    sim.depth_update();
    double maxdepth_after = sim.maxdepth;
    sim.check_wetted_area(scan_area_interval_iter);
    if (!sim.is_hydro_only()) {
      sim.call_erosion();
      if (lateral) sim.call_lateral();
    }
    sim.water_flux_out();
    sim.call_channel_landsliding(in_channel_landslide_iter_interval);
    if (!nohill) {
      sim.slope_creep(creep_time_interval_days, creep_coeff);
      sim.call_global_landsliding(global_landsliding_interval_hours);
    }
    sim.grow_vegetation(vegetation_growth_interval_hours);
    double rec[10] = {(double)sim.counter, sim.cycle,        sim.time_step,
                      maxdepth_after,      sim.waterOut,     sim.waterinput,
                      sim.erode_mult,      sim.sediQ,        sim.globalsediq,
                      sim.baseflow};
    std::fwrite(rec, sizeof(double), 10, steps);
    it++;
    if (iters >= 0 && it >= iters) break;
  } while (sim.get_cycle() / 60 < sim.get_maxcycle());
  auto t1 = std::chrono::steady_clock::now();
  std::fclose(steps);

  Dump d{std::fopen(outfn.c_str(), "wb")};
  d.arr2("elev", 'd', sim.elev);
  d.arr2("water_depth", 'd', sim.water_depth);
  d.arr2("qx", 'd', sim.qx);
  d.arr2("qy", 'd', sim.qy);
  d.arr2("qxs", 'd', sim.qxs);
  d.arr2("qys", 'd', sim.qys);
  d.arr2("Vsusptot", 'd', sim.Vsusptot);
  d.arr2("Vel", 'd', sim.Vel);
  d.arr2("Tau", 'd', sim.Tau);
  d.arr2("bedrock", 'd', sim.bedrock);
  d.arr2("area", 'd', sim.area);
  d.arr2("index", 'i', sim.index);
  d.arr2("down_scan", 'i', sim.down_scan);
  d.arr2("edge", 'd', sim.edge);
  d.arr3("vel_dir", 'd', sim.vel_dir);
  if (!sim.hydro_only) {
    d.arr2("grain", 'd', sim.grain);
    d.arr3("strata", 'd', sim.strata);
    d.arr3("sr", 'd', sim.sr);
    d.arr3("sl", 'd', sim.sl);
    d.arr3("su", 'd', sim.su);
    d.arr3("sd", 'd', sim.sd);
    d.arr2("ss", 'd', sim.ss);
  }
  d.dbl("cycle", sim.cycle);
  d.dbl("time_step", sim.time_step);
  d.dbl("maxdepth", sim.maxdepth);
  d.dbl("waterOut", sim.waterOut);
  d.dbl("waterinput", sim.waterinput);
  d.dbl("counter", sim.counter);
  d.dbl("grain_array_tot", sim.grain_array_tot);
  d.dbl("erode_mult", sim.erode_mult);
  d.dbl("erode_call", sim.erode_call);
  d.dbl("sediQ", sim.sediQ);
  d.dbl("globalsediq", sim.globalsediq);
  d.dbl("baseflow", sim.baseflow);
  d.dbl("totalinputpoints", sim.totalinputpoints);
  d.dbl("time_1", sim.time_1);
  d.dbl("lateralcounter", sim.lateralcounter);
  d.dbl("step_seconds", std::chrono::duration<double>(t1 - t0).count());
  d.dbl("iterations", (double)it);
  for (unsigned n = 1; n <= sim.G_MAX; n++) {
    char nm[32];
    std::snprintf(nm, sizeof nm, "sum_grain%u", n);
    d.dbl(nm, sim.sum_grain[n]);
  }
  std::fclose(d.f);
  return 0;
}
