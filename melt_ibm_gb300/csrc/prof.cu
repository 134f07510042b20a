// prof.cu -- per-kernel CUDA-event profiling of the bound context.
//
// The reference's TIMED build brackets each substep phase with barriers and
// wall clocks (tsch.f90:26-84, mpi_routines.f90:2346-2361).  Here, when
// profiling is switched on, every instrumented launch is bracketed by two
// CUDA events on the context stream; totals per kernel name are read back
// with mibm_profile_get_.  Off by default (no events recorded).
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"

namespace mibm {

struct ProfRec {
  std::string name;
  cudaEvent_t a, b;
};

struct ProfState {
  bool on = false;
  std::vector<ProfRec> recs;
  size_t used = 0;
  std::vector<std::pair<std::string, std::pair<double, long>>> table;  // name -> (ms, launches)
};

static std::map<Ctx*, ProfState> g_prof;

ProfScope::ProfScope(Ctx* c, const char* name) : c_(c), idx_(-1) {
  auto it = g_prof.find(c);
  if (it == g_prof.end() || !it->second.on) return;
  ProfState& s = it->second;
  if (s.used == s.recs.size()) {
    ProfRec r;
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    s.recs.push_back(r);
  }
  idx_ = (int)s.used++;
  s.recs[idx_].name = name;
  cudaEventRecord(s.recs[idx_].a, c->stream);
}

ProfScope::~ProfScope() {
  if (idx_ < 0) return;
  cudaEventRecord(g_prof[c_].recs[idx_].b, c_->stream);
}

static void collect(Ctx* c) {
  ProfState& s = g_prof[c];
  if (s.used == 0) return;
  cudaStreamSynchronize(c->stream);
  for (size_t q = 0; q < s.used; ++q) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s.recs[q].a, s.recs[q].b);
    bool found = false;
    for (auto& e : s.table)
      if (e.first == s.recs[q].name) { e.second.first += ms; e.second.second += 1; found = true; break; }
    if (!found) s.table.push_back({s.recs[q].name, {(double)ms, 1L}});
  }
  s.used = 0;
}

void prof_release(Ctx* c) {
  auto it = g_prof.find(c);
  if (it == g_prof.end()) return;
  for (auto& r : it->second.recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  g_prof.erase(it);
}

// Recording more than this many launches between two reads flushes the
// pending records into the totals (bounded event pool).
void prof_flush_if_full(Ctx* c) {
  auto it = g_prof.find(c);
  if (it != g_prof.end() && it->second.used > 4096) collect(c);
}

}  // namespace mibm

using namespace mibm;

extern "C" {

// on != 0 starts (and clears) profiling of the bound context; 0 stops it.
void mibm_profile_(const int* on) {
  Ctx* c = current(); if (!c) return;
  ProfState& s = g_prof[c];
  if (*on) { collect(c); s.table.clear(); s.on = true; }
  else { collect(c); s.on = false; }
  c->profiling = s.on;
}

// Number of distinct kernel names recorded so far (collects pending events).
int mibm_profile_count_(void) {
  Ctx* c = current(); if (!c) return 0;
  collect(c);
  return (int)g_prof[c].table.size();
}

// Entry `idx`: name (NUL-terminated, truncated to `cap`), total ms, launches.
int mibm_profile_get_(const int* idx, char* name, const int* cap, double* total_ms, long long* launches) {
  Ctx* c = current(); if (!c) return MIBM_ESTATE;
  ProfState& s = g_prof[c];
  if (*idx < 0 || *idx >= (int)s.table.size()) return MIBM_EINVAL;
  const auto& e = s.table[*idx];
  std::strncpy(name, e.first.c_str(), (size_t)*cap);
  if (*cap > 0) name[*cap - 1] = 0;
  *total_ms = e.second.first;
  *launches = e.second.second;
  return MIBM_OK;
}

}  // extern "C"
