#include "profile.hpp"

#include <cstdio>
#include <map>
#include <mutex>
#include <vector>

namespace pgpu {

namespace {

struct Rec {
  std::string name;
  cudaEvent_t beg = nullptr, end = nullptr;
  double flops = 0, bytes = 0;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;

}  // namespace

bool profile_enabled() { return g_on; }

void profile_enable(bool on) { g_on = on; }

void profile_reset() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_recs) {
    if (r.beg) cudaEventDestroy(r.beg);
    if (r.end) cudaEventDestroy(r.end);
  }
  g_recs.clear();
}

std::string profile_report() {
  sync();
  std::lock_guard<std::mutex> lk(g_mu);
  struct Agg {
    long calls = 0;
    double ms = 0, flops = 0, bytes = 0;
  };
  std::map<std::string, Agg> agg;
  for (auto& r : g_recs) {
    float ms = 0;
    if (r.beg && r.end && cudaEventElapsedTime(&ms, r.beg, r.end) != cudaSuccess) {
      cudaGetLastError();
      ms = 0;
    }
    auto& a = agg[r.name];
    a.calls++;
    a.ms += ms;
    a.flops += r.flops;
    a.bytes += r.bytes;
  }
  std::string out = "{";
  bool first = true;
  for (auto& [k, a] : agg) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s\"%s\": {\"calls\": %ld, \"ms\": %.6f, \"flops\": %.6e, \"bytes\": %.6e}",
                  first ? "" : ", ", k.c_str(), a.calls, a.ms, a.flops, a.bytes);
    out += buf;
    first = false;
  }
  out += "}";
  return out;
}

ProfScope::ProfScope(const char* name, double flops, double bytes) {
  if (!g_on) return;
  Rec r;
  r.name = name;
  r.flops = flops;
  r.bytes = bytes;
  PGPU_CUDA(cudaEventCreate(&r.beg));
  PGPU_CUDA(cudaEventCreate(&r.end));
  PGPU_CUDA(cudaEventRecord(r.beg, stream()));
  std::lock_guard<std::mutex> lk(g_mu);
  slot_ = static_cast<int>(g_recs.size());
  g_recs.push_back(r);
}

ProfScope::~ProfScope() {
  if (slot_ < 0) return;
  cudaEvent_t e;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    e = g_recs[slot_].end;
  }
  cudaEventRecord(e, stream());
}

}  // namespace pgpu
