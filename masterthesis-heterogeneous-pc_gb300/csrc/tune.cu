// Process-wide table of CI-test tile policies, keyed by (largest p of a launch,
// level, largest degree at the level start), each key a bit-length bucket. The
// autotuner (hpc_autotune, ctx.cu) fills it from measured level-kernel times; contexts
// copy it to the device before a run and every level kernel reads its entry after the
// test-count scan. No counterpart in the reference, whose launch shapes are fixed
// (src/executor/gpuExecutor.cu:45-106: one 64-thread block per row and neighbour slot).
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.cuh"

namespace hpc {
namespace {

constexpr int kLv = HPC_MAX_LEVEL + 1;
std::mutex g_mu;
std::vector<TuneEntry> g_table((size_t)kTunePB * kLv * kTuneDB);  // tile_cap 0 = no entry
long long g_version = 1;

size_t index_of(int pb, int level, int db) { return ((size_t)pb * kLv + level) * kTuneDB + db; }

bool valid_params(const hpc_tune_params &p) {
  return p.tile_cap >= 1 && p.tile_cap <= kTuneMaxCap && p.tiles_per_lane >= 1 && p.tiles_per_lane <= 64 &&
         (p.edge_lanes == 1 || p.edge_lanes == 32) && (p.l1_prefetch == 0 || p.l1_prefetch == 1);
}

hpc_status check_key(int64_t p, int level, int max_degree) {
  if (p < 2 || level < 1 || level > HPC_MAX_LEVEL || max_degree < 0) {
    set_error("tile-policy key needs p >= 2, 1 <= level <= %d, max_degree >= 0", HPC_MAX_LEVEL);
    return HPC_ERR_INVALID_ARG;
  }
  return HPC_OK;
}

}  // namespace

TuneEntry tune_entry_of(const hpc_tune_params &p) {
  return TuneEntry{p.tile_cap, p.tiles_per_lane, p.edge_lanes, p.l1_prefetch};
}

bool tune_params_valid(const hpc_tune_params *p) { return p && valid_params(*p); }

void tune_snapshot(std::vector<TuneEntry> *out, long long *version) {
  std::lock_guard<std::mutex> g(g_mu);
  *out = g_table;
  *version = g_version;
}

long long tune_version() {
  std::lock_guard<std::mutex> g(g_mu);
  return g_version;
}

TuneEntry tune_get(int p_bucket, int level, int deg_bucket) {
  std::lock_guard<std::mutex> g(g_mu);
  return g_table[index_of(p_bucket, level, deg_bucket)];
}

void tune_store(int64_t p, int level, int max_degree, const TuneEntry &e) {
  std::lock_guard<std::mutex> g(g_mu);
  g_table[index_of(tune_bucket(p, kTunePB), level, tune_bucket(max_degree, kTuneDB))] = e;
  ++g_version;
}

}  // namespace hpc

using namespace hpc;

extern "C" {

hpc_status hpc_tune_set(int64_t p, int level, int max_degree, const hpc_tune_params *prm) {
  hpc_status s = check_key(p, level, max_degree);
  if (s != HPC_OK) return s;
  if (prm && !valid_params(*prm)) {
    set_error("tile policy needs 1 <= tile_cap <= %d, 1 <= tiles_per_lane <= 64, edge_lanes 1 or 32, l1_prefetch 0 or 1",
              kTuneMaxCap);
    return HPC_ERR_INVALID_ARG;
  }
  tune_store(p, level, max_degree, prm ? tune_entry_of(*prm) : TuneEntry{0, 0, 0, 0});
  return HPC_OK;
}

hpc_status hpc_tune_lookup(int64_t p, int level, int max_degree, hpc_tune_params *out, int *found) {
  hpc_status s = check_key(p, level, max_degree);
  if (s != HPC_OK) return s;
  if (!out) {
    set_error("null output pointer");
    return HPC_ERR_INVALID_ARG;
  }
  TuneEntry e;
  {
    std::lock_guard<std::mutex> g(g_mu);
    e = g_table[index_of(tune_bucket(p, kTunePB), level, tune_bucket(max_degree, kTuneDB))];
  }
  const bool have = e.tile_cap > 0;
  out->tile_cap = have ? e.tile_cap : kTuneDefaultCap;
  out->tiles_per_lane = have ? e.tiles_per_lane : kTuneDefaultTpl;
  out->edge_lanes = have ? e.edge_lanes : kTuneDefaultEdgeLanes;
  out->l1_prefetch = have ? e.l1_prefetch : 0;
  if (found) *found = have ? 1 : 0;
  return HPC_OK;
}

hpc_status hpc_tune_clear(void) {
  std::lock_guard<std::mutex> g(g_mu);
  std::fill(g_table.begin(), g_table.end(), TuneEntry{0, 0, 0, 0});
  ++g_version;
  return HPC_OK;
}

// Text file: a header line, then one line per entry:
//   p_bucket level degree_bucket tile_cap tiles_per_lane edge_lanes l1_prefetch
hpc_status hpc_tune_save(const char *path) {
  if (!path) {
    set_error("null path");
    return HPC_ERR_INVALID_ARG;
  }
  std::vector<TuneEntry> t;
  long long v;
  tune_snapshot(&t, &v);
  FILE *f = std::fopen(path, "w");
  if (!f) {
    set_error("cannot write %s", path);
    return HPC_ERR_INVALID_ARG;
  }
  std::fprintf(f, "heterogpc-tile-policy 2 %d %d %d\n", kTunePB, kLv, kTuneDB);
  for (int pb = 0; pb < kTunePB; ++pb)
    for (int l = 0; l < kLv; ++l)
      for (int db = 0; db < kTuneDB; ++db) {
        const TuneEntry &e = t[index_of(pb, l, db)];
        if (e.tile_cap > 0)
          std::fprintf(f, "%d %d %d %d %d %d %d\n", pb, l, db, e.tile_cap, e.tiles_per_lane, e.edge_lanes, e.l1_prefetch);
      }
  const bool ok = std::fclose(f) == 0;
  if (!ok) {
    set_error("error writing %s", path);
    return HPC_ERR_INVALID_ARG;
  }
  return HPC_OK;
}

// Entries of the file are added to the table (replacing entries of the same key).
hpc_status hpc_tune_load(const char *path) {
  if (!path) {
    set_error("null path");
    return HPC_ERR_INVALID_ARG;
  }
  FILE *f = std::fopen(path, "r");
  if (!f) {
    set_error("cannot read %s", path);
    return HPC_ERR_INVALID_ARG;
  }
  int ver = 0, npb = 0, nl = 0, ndb = 0;
  if (std::fscanf(f, "heterogpc-tile-policy %d %d %d %d", &ver, &npb, &nl, &ndb) != 4 || ver != 2 ||
      npb != kTunePB || nl != kLv || ndb != kTuneDB) {
    std::fclose(f);
    set_error("%s is not a tile-policy file of this library", path);
    return HPC_ERR_INVALID_ARG;
  }
  std::vector<std::pair<size_t, TuneEntry>> rows;
  int pb, l, db, cap, tpl, l1, pf;
  int r;
  while ((r = std::fscanf(f, "%d %d %d %d %d %d %d", &pb, &l, &db, &cap, &tpl, &l1, &pf)) == 7) {
    const hpc_tune_params prm{cap, tpl, l1, pf};
    if (pb < 0 || pb >= kTunePB || l < 1 || l >= kLv || db < 0 || db >= kTuneDB || !valid_params(prm)) {
      std::fclose(f);
      set_error("%s: bad entry %d %d %d %d %d %d %d", path, pb, l, db, cap, tpl, l1, pf);
      return HPC_ERR_INVALID_ARG;
    }
    rows.push_back({index_of(pb, l, db), tune_entry_of(prm)});
  }
  const bool clean_end = r == EOF;
  std::fclose(f);
  if (!clean_end) {
    set_error("%s: malformed line", path);
    return HPC_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> g(g_mu);
  for (const auto &e : rows) g_table[e.first] = e.second;
  ++g_version;
  return HPC_OK;
}

}  // extern "C"
