// Host check of the C++ facade (include/idefix_gb300.hpp) against a scripted
// fake of the C ABI defined below: the reference-named calls forward to the
// right entry points in the reference's order, with the block's t and dt
// where the reference passes them, results come back, every non-zero status
// becomes an idefix_gb300::Error (a std::runtime_error) with the status and
// the handle's message, and the handle is destroyed exactly once.  Prints
// "facade ok" and exits 0 when every check holds.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/idefix_gb300.hpp"

// ---- fake C ABI ------------------------------------------------------------
struct idfx_gpu {
  int id;
};
static std::vector<std::string> g_log;
static int g_next_status = IDFX_OK;  // status returned by the next scripted call
static int g_created = 0, g_destroyed = 0;
static double g_t = 0.25, g_dt = 1e-3;
static long long g_ncycles = 0;

static int scripted(const std::string& call) {
  g_log.push_back(call);
  const int st = g_next_status;
  g_next_status = IDFX_OK;
  return st;
}

extern "C" {
int idfx_gpu_create(const idfx_gpu_config* cfg, void*, idfx_gpu** out) {
  *out = nullptr;
  const int st = scripted("create");
  if (st == IDFX_OK) {
    *out = new idfx_gpu{cfg->dims};
    g_created++;
  }
  return st;
}
int idfx_gpu_destroy(idfx_gpu* h) {
  g_log.push_back("destroy");
  g_destroyed++;
  delete h;
  return IDFX_OK;
}
int idfx_gpu_last_error(const idfx_gpu*, char* buf, size_t len) {
  std::snprintf(buf, len, "%s", "NaN in RHO at cell (3, 4, 0)");
  return IDFX_OK;
}
int idfx_gpu_upload_prim(idfx_gpu*, const double*, const double*) { return scripted("upload_prim"); }
int idfx_gpu_download_prim(idfx_gpu*, double*, double*) { return scripted("download_prim"); }
int idfx_gpu_download_cons(idfx_gpu*, double*) { return scripted("download_cons"); }
int idfx_gpu_upload_prim_device(idfx_gpu*, const double*, const double*) { return scripted("upload_prim_device"); }
int idfx_gpu_download_prim_device(idfx_gpu*, double*, double*) { return scripted("download_prim_device"); }
int idfx_gpu_set_time(idfx_gpu*, double t, double dt, long long n) {
  g_t = t, g_dt = dt, g_ncycles = n;
  return scripted("set_time");
}
int idfx_gpu_get_time(idfx_gpu*, double* t, double* dt, long long* n) {
  if (t) *t = g_t;
  if (dt) *dt = g_dt;
  if (n) *n = g_ncycles;
  return IDFX_OK;
}
int idfx_gpu_cycle(idfx_gpu*) {
  const int st = scripted("cycle");
  if (st == IDFX_OK) g_ncycles++;
  return st;
}
int idfx_gpu_run(idfx_gpu*, double tstop, long long max_cycles) {
  return scripted("run " + std::to_string(tstop) + " " + std::to_string(max_cycles));
}
int idfx_gpu_set_boundaries(idfx_gpu*) { return scripted("set_boundaries"); }
int idfx_gpu_prim_to_cons(idfx_gpu*) { return scripted("prim_to_cons"); }
int idfx_gpu_cons_to_prim(idfx_gpu*) { return scripted("cons_to_prim"); }
int idfx_gpu_reset_stage(idfx_gpu*) { return scripted("reset_stage"); }
int idfx_gpu_evolve_stage(idfx_gpu*, double t, double dt) {
  char b[96];
  std::snprintf(b, sizeof(b), "evolve_stage %.17g %.17g", t, dt);
  return scripted(b);
}
int idfx_gpu_compute_timestep(idfx_gpu*, double* dt) {
  *dt = 2.5e-3;
  return scripted("compute_timestep");
}
int idfx_gpu_check_divb(idfx_gpu*, double* v) {
  *v = 3.0e-15;
  return scripted("check_divb");
}
int idfx_gpu_check_nan(idfx_gpu*, long long* n) {
  *n = 7;
  return scripted("check_nan");
}
}  // extern "C"

// ---- checks ----------------------------------------------------------------
static int g_fail = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAILED line %d: %s\n", __LINE__, #c);          \
      g_fail++;                                                   \
    }                                                             \
  } while (0)

int main() {
  namespace ig = idefix_gb300;
  idfx_gpu_config cfg{};
  cfg.dims = 2;

  {  // the reference's stage sequence through reference-named calls
    ig::DataBlock data(cfg);
    ig::TimeIntegrator tint;
    data.block.SetTime(0.5, 1e-4, 0);
    data.hydro->ResetStage();
    data.hydro->boundary->SetBoundaries(0.5);
    data.hydro->ConvertPrimToCons();
    data.EvolveStage();
    data.hydro->ConvertConsToPrim();
    const double dt = data.ComputeTimestep();
    CHECK(dt == 2.5e-3);
    CHECK(data.hydro->CheckDivB() == 3.0e-15);
    CHECK(data.hydro->CheckNan() == 7);
    tint.Cycle(data);
    tint.Cycle(data);
    CHECK(tint.GetNCycles(data) == 2);
    tint.Run(data, 1.0);
    const std::vector<std::string> want = {
        "create", "set_time", "reset_stage", "set_boundaries", "prim_to_cons",
        "evolve_stage 0.5 0.0001", "cons_to_prim", "compute_timestep", "check_divb", "check_nan",
        "cycle", "cycle", "run 1.000000 -1"};
    CHECK(g_log == want);
    if (g_log != want)
      for (auto& s : g_log) std::printf("  logged: %s\n", s.c_str());
  }
  CHECK(g_created == 1 && g_destroyed == 1);

  {  // a refused setup: Error with the status, no handle to destroy
    g_next_status = IDFX_ERR_CONFIG;
    bool thrown = false;
    try {
      ig::DataBlock data(cfg);
    } catch (const ig::Error& e) {
      thrown = true;
      CHECK(e.status() == IDFX_ERR_CONFIG);
      CHECK(!e.numerical());
      CHECK(std::strstr(e.what(), "invalid setup") != nullptr);
    }
    CHECK(thrown);
    CHECK(g_created == 1 && g_destroyed == 1);
  }

  {  // a numerical failure reaches main's catch (std::runtime_error), with the message
    ig::DataBlock data(cfg);
    ig::TimeIntegrator tint;
    g_next_status = IDFX_ERR_NAN;
    bool thrown = false;
    try {
      tint.Cycle(data);
    } catch (const std::runtime_error& e) {
      thrown = true;
      const ig::Error* ie = dynamic_cast<const ig::Error*>(&e);
      CHECK(ie && ie->status() == IDFX_ERR_NAN && ie->numerical());
      CHECK(std::strstr(e.what(), "Cycle") != nullptr);
      CHECK(std::strstr(e.what(), "NaN in RHO") != nullptr);
    }
    CHECK(thrown);
    for (int st : {IDFX_ERR_DIVB, IDFX_ERR_DT_SMALL}) {
      g_next_status = st;
      try {
        tint.Cycle(data);
        CHECK(false);
      } catch (const ig::Error& e) {
        CHECK(e.status() == st && e.numerical());
      }
    }
    for (int st : {IDFX_ERR_FIRST_DT, IDFX_ERR_CUDA, IDFX_ERR_STATE}) {
      g_next_status = st;
      try {
        data.hydro->EvolveStage(0.0, 1e-3);
        CHECK(false);
      } catch (const ig::Error& e) {
        CHECK(e.status() == st && !e.numerical());
      }
    }
  }
  CHECK(g_created == 2 && g_destroyed == 2);

  {  // moving a block hands over the handle; it is destroyed once
    ig::Block a(cfg);
    ig::Block b(std::move(a));
    CHECK(a.handle() == nullptr && b.handle() != nullptr);
    ig::Block c(cfg);
    c = std::move(b);
    CHECK(g_destroyed == 3);  // c's own handle
  }
  CHECK(g_created == 4 && g_destroyed == 4);

  if (g_fail == 0) std::printf("facade ok\n");
  return g_fail != 0;
}
