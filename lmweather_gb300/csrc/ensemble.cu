// Ensembles of spheres with mixed truncations: one engine per truncation, its members stacked along the batch
// dimension of every kernel (the member axis becomes the M dimension of the split-precision GEMMs), each engine
// on its own stream. A run plans every group at its own stable step (the reference's stable_dt(1.5), the
// smallest over the group's members, cpp/sphere.cpp:438-447) and interleaves the groups' 64-step graph chunks,
// checking each group's guards (cpp/sphere.cpp:473-483) at its guard points.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>

#include "engine.h"

namespace lmw {

EnsembleEngine::EnsembleEngine(const std::vector<MemberSpec> &specs, double radius, double gravity, double max_wind, int precision,
                               int split_terms)
    : members(specs) {
  if (specs.empty()) throw InvalidArgument("an ensemble needs at least one member");
  std::map<int, std::vector<int>> by_t;
  for (size_t i = 0; i < specs.size(); i++) {
    const MemberSpec &m = specs[i];
    if (m.truncation < 4 || m.truncation > 341) throw InvalidArgument("truncation must be between 4 and 341");
    if (!(m.mean_height > 0)) throw InvalidArgument("mean height must be positive");
    by_t[m.truncation].push_back(static_cast<int>(i));
  }
  group_of.assign(specs.size(), 0);
  index_in_group.assign(specs.size(), 0);
  for (auto &kv : by_t) {
    const int T = kv.first;
    SphereConfig c;
    c.truncation = T;
    c.radius = radius;
    c.gravity = gravity;
    c.omega = specs[kv.second[0]].omega;
    // del^4 diffusion with a 1-day e-folding at the truncation wavenumber (the benchmark recipe)
    c.diffusion = std::pow(radius, 4) / (86400.0 * std::pow(T * (T + 1.0), 2));
    c.precision = precision;
    c.split_terms = split_terms;
    c.members = static_cast<int>(kv.second.size());
    c.max_truncation = 341;
    auto eng = std::make_unique<SphereEngine>(c);
    for (size_t k = 0; k < kv.second.size(); k++) {
      const int i = kv.second[k];
      group_of[i] = static_cast<int>(groups.size());
      index_in_group[i] = static_cast<int>(k);
      eng->set_omega(specs[i].omega, static_cast<int>(k));
      eng->turbulence(specs[i].seed, specs[i].mean_height, max_wind, T / 2, static_cast<int>(k));
    }
    truncations.push_back(T);
    groups.push_back(std::move(eng));
  }
  last_dt.assign(groups.size(), 0.0);
  last_steps.assign(groups.size(), 0);
}

void EnsembleEngine::run(double seconds) {
  const size_t G = groups.size();
  std::vector<SphereEngine::RunPlan> plans(G);
  for (size_t g = 0; g < G; g++) {
    plans[g] = groups[g]->plan_run(seconds, 0.0);
    last_dt[g] = plans[g].h;
    last_steps[g] = plans[g].n;
  }
  bool any = true;
  std::vector<char> moved(G);
  while (any) {
    any = false;
    for (size_t g = 0; g < G; g++) {
      moved[g] = groups[g]->advance(plans[g]) ? 1 : 0;
      any = any || moved[g];
    }
    for (size_t g = 0; g < G; g++)
      if (moved[g]) groups[g]->guard(plans[g]);
  }
}

// Runs of consecutive members in one group with consecutive indices in it: one copy per run and field.
template <class F> static void for_runs(const EnsembleEngine &e, F &&fn) {
  const int n = static_cast<int>(e.members.size());
  size_t off = 0;  // complex values before member i in each field
  for (int i = 0; i < n;) {
    int j = i + 1;
    while (j < n && e.group_of[j] == e.group_of[i] && e.index_in_group[j] == e.index_in_group[j - 1] + 1) j++;
    const size_t mm = static_cast<size_t>(e.truncations[e.group_of[i]] + 1) * (e.truncations[e.group_of[i]] + 1);
    fn(e.group_of[i], e.index_in_group[i], j - i, off, mm);
    off += mm * (j - i);
    i = j;
  }
}

void EnsembleEngine::get_states(double *zeta, double *delta, double *phi) {
  std::vector<double *> dev(groups.size());
  for (size_t g = 0; g < groups.size(); g++) dev[g] = groups[g]->states_to_ref();
  double *out[3] = {zeta, delta, phi};
  for_runs(*this, [&](int g, int k0, int cnt, size_t off, size_t mm) {
    SphereEngine &s = *groups[g];
    for (int f = 0; f < 3; f++)
      LMW_CUDA(cudaMemcpyAsync(out[f] + 2 * off, dev[g] + 2 * ((static_cast<size_t>(f) * s.B + k0) * mm), cnt * mm * 2 * sizeof(double),
                               cudaMemcpyDeviceToHost, s.stream));
  });
  for (auto &g : groups) LMW_CUDA(cudaStreamSynchronize(g->stream));
}

void EnsembleEngine::set_states(const double *zeta, const double *delta, const double *phi) {
  std::vector<double *> dev(groups.size());
  for (size_t g = 0; g < groups.size(); g++) {
    LMW_CUDA(cudaStreamSynchronize(groups[g]->stream));
    dev[g] = groups[g]->device_refstates();
  }
  const double *in[3] = {zeta, delta, phi};
  for_runs(*this, [&](int g, int k0, int cnt, size_t off, size_t mm) {
    SphereEngine &s = *groups[g];
    for (int f = 0; f < 3; f++)
      LMW_CUDA(cudaMemcpyAsync(dev[g] + 2 * ((static_cast<size_t>(f) * s.B + k0) * mm), in[f] + 2 * off, cnt * mm * 2 * sizeof(double),
                               cudaMemcpyHostToDevice, s.stream));
  });
  for (auto &g : groups) g->states_from_ref();
  for (auto &g : groups) LMW_CUDA(cudaStreamSynchronize(g->stream));
}

void EnsembleEngine::check_member(int i) const {
  if (i < 0 || i >= static_cast<int>(members.size())) throw InvalidArgument("member index out of range");
}

}  // namespace lmw
