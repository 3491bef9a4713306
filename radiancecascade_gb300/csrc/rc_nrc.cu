// rc_nrc.cu -- the neural radiance cache of include/rc.h: state, the
// per-solve schedule (training-sample walks, held-out error, refit, inference,
// fallback, merges) and the rc_nrc_* entry points.
//
// Reference boundary: the learned form is an engine option behind the same
// solve; the reference's GI stage (src/app.rs:3-7) sees no difference.

#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "rc_ctx.h"
#include "rc_nrc.cuh"

static_assert(RC_MAX_CASCADES == rcx::kMaxCascades, "rc_nrc_stats.served_solves covers every cascade");

namespace rcx {

struct NrcState {
  rc_nrc_params prm{};
  int first = 2, nlev = 0, nph = 16;
  int64_t T = 0;       // entries per hash level
  int64_t hash_n = 0;  // 16 * T * 2
  float *hash_master = nullptr, *hash_m = nullptr, *hash_v = nullptr, *hash_g = nullptr;
  __half* hash_half = nullptr;
  float *mlp = nullptr, *mlp_m = nullptr, *mlp_v = nullptr, *mlp_g = nullptr, *dbg_g = nullptr;
  unsigned char* img = nullptr;
  __nv_bfloat16* denc = nullptr;
  __half* rt = nullptr;
  int64_t enum_tiles = 0;
  // sample tiles grouped by phase: every far probe with the directions of the
  // phase (rows of up to 128; short direction lists pack several probes); a
  // tile's slot is its first probe's index in the phase
  NrcTile* tiles = nullptr;
  std::vector<NrcTile> h_tiles;
  std::vector<uint8_t> probe_tile;  // tiles that hold a far probe
  std::vector<int64_t> tile_begin;
  int32_t* dlist = nullptr;  // directions of the sample tiles, per level and phase
  int64_t dlist_base[kMaxCascades]{};  // a level's directions in dlist
  // per level and phase pair q: start (in the level's directions) and length
  // of the run of phases q and q + nph/2 in dlist
  std::vector<std::vector<int64_t>> pair_start = std::vector<std::vector<int64_t>>(kMaxCascades),
                                    pair_len = std::vector<std::vector<int64_t>>(kMaxCascades);
  int64_t max_tiles2 = 0, max_held = 0;
  float* target = nullptr;
  float* pred = nullptr;
  float* epos_grad = nullptr;
  float* loss = nullptr;
  float* h_loss = nullptr;    // pinned
  unsigned* count = nullptr;  // probes in fallback tiles per far level
  int32_t* plain = nullptr;   // per level: 1 = the level runs on its walks this solve
  unsigned long long* served_solves = nullptr;  // per level: solves the network served it
  int64_t total_probes = 0;
  NrcTile* qtiles = nullptr;  // rc_nrc_query / rc_nrc_tile_gradient scratch
  float* qout = nullptr;
  int64_t qcap = 0;
  // the far levels' own walk queue: records, step tables, per-word switches
  QueueArgs fq{};
  uint32_t* frec = nullptr;
  unsigned long long* fcounter = nullptr;
  uint2* fsteps = nullptr;
  int32_t* fstep_begin = nullptr;
  bool ftab = false;
  int fq_resident = 0;  // walk blocks that fit the GPU at once
  uint8_t* word_on = nullptr;
  float* omega = nullptr;
  uint32_t* hparts = nullptr;  // hash parts of the far probes, then of the far directions
  NrcWordArgs words{};
  // fallback tiles
  int tile_shift = 3, TX = 0, TY = 0, TZ = 0;
  float *tnum = nullptr, *tden = nullptr, *tring = nullptr;
  uint8_t* flag = nullptr;
  NrcArgs base{};
  int64_t solves = 0, steps = 0;
  int64_t loss_rows = 0;
  int fwd_blocks = 0, train_blocks = 0;
};

namespace {

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
float uniform(uint64_t& s, float lo, float hi) {
  return lo + (hi - lo) * (float)((splitmix(s) >> 11) * (1.0 / 9007199254740992.0));
}

void free_state(NrcState* n) {
  if (!n) return;
  void* bufs[] = {n->hash_master, n->hash_m, n->hash_v, n->hash_g, n->hash_half, n->mlp,   n->mlp_m,
                  n->mlp_v,       n->mlp_g,  n->dbg_g,  n->img,    n->denc,      n->rt,    n->tiles,
                  n->dlist, n->target, n->pred,   n->epos_grad, n->loss,  n->qtiles,
                  n->qout,        n->tnum,   n->tden,   n->tring,   n->flag,   n->count,     n->plain, n->served_solves, n->frec,
                  n->fcounter,    n->fsteps, n->fstep_begin, n->word_on, n->omega, n->hparts};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (n->h_loss) cudaFreeHost(n->h_loss);
  delete n;
}

rc_status check(const rc_context* c, const char* fn, bool need_nrc) {
  if (!c) {
    set_error("%s: context is NULL", fn);
    return RC_ERR_INVALID_ARG;
  }
  if (need_nrc && !c->nrc) {
    set_error("%s: the radiance cache is not enabled", fn);
    return RC_ERR_STATE;
  }
  return RC_OK;
}

unsigned blocks_for(int64_t n, int threads) { return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads); }

// count is a multiple of 4 (the MLP's 17,680 parameters, the hash table's 32 T).
void launch_adam(float* p, float* g, float* m, float* v, __half* half_out, int64_t count, const rc_nrc_params& prm,
                 int64_t t, bool lazy, cudaStream_t s) {
  AdamArgs a;
  a.lazy = lazy ? 1 : 0;
  a.pad = 0;
  a.p = p;
  a.g = g;
  a.m = m;
  a.v = v;
  a.half_out = half_out;
  a.n = count;
  a.lr = prm.learning_rate;
  a.beta1 = prm.beta1;
  a.beta2 = prm.beta2;
  a.eps = prm.epsilon;
  a.c1 = (float)(1.0 - pow((double)prm.beta1, (double)t));
  a.c2 = (float)(1.0 - pow((double)prm.beta2, (double)t));
  k_nrc_adam<<<(unsigned)std::min<int64_t>(blocks_for(count / 4, 256), 152 * 8), 256, 0, s>>>(a);
}

void launch_pack(NrcState* n, cudaStream_t s) {
  k_nrc_pack<<<blocks_for(kImgBytes / 2, 256), 256, 0, s>>>(n->mlp, n->img);
}

rc_status ensure_query(NrcState* n, int64_t count) {
  if (count <= n->qcap) return RC_OK;
  if (n->qtiles) cudaFree(n->qtiles);
  if (n->qout) cudaFree(n->qout);
  n->qtiles = nullptr;
  n->qout = nullptr;
  n->qcap = 0;
  rc_status s = dev_alloc((void**)&n->qtiles, count * sizeof(NrcTile), "cache query tiles");
  if (s != RC_OK) return s;
  if ((s = dev_alloc((void**)&n->qout, count * kNrcThreads * 4 * sizeof(float), "cache query output")) != RC_OK)
    return s;
  n->qcap = count;
  return RC_OK;
}

void init_params(NrcState* n, std::vector<float>& mlp, std::vector<float>& hash) {
  uint64_t s = n->prm.seed;
  mlp.assign(kNrcParams, 0.f);
  for (int l = 0; l < kNrcHidden; ++l) {
    const int fan_in = l == 0 ? kNrcPosFeat + kNrcDirFeat : 64;
    const float r = sqrtf(6.f / (float)fan_in);
    float* W = mlp.data() + l * kNrcLayerStride;
    for (int o = 0; o < 64; ++o)
      for (int i = 0; i < 64; ++i) W[o * 64 + i] = (l == 0 && i >= fan_in) ? 0.f : uniform(s, -r, r);
  }
  const float r4 = sqrtf(6.f / 64.f) * 0.1f;
  for (int o = 0; o < 4; ++o)
    for (int i = 0; i < 64; ++i) mlp[kNrcW4 + o * 64 + i] = uniform(s, -r4, r4);
  hash.resize((size_t)n->hash_n);
  for (auto& v : hash) v = uniform(s, -1e-4f, 1e-4f);
}

rc_status upload_params(NrcState* n, const std::vector<float>& mlp, const std::vector<float>& hash) {
  RC_CUDA(check_prepare(), "checked build: range upload");
  RC_CUDA(cudaMemcpy(n->mlp, mlp.data(), mlp.size() * 4, cudaMemcpyHostToDevice), "cache upload");
  RC_CUDA(cudaMemcpy(n->hash_master, hash.data(), hash.size() * 4, cudaMemcpyHostToDevice), "cache upload");
  std::vector<__half> hh(hash.size());
  for (size_t i = 0; i < hash.size(); ++i) hh[i] = __float2half_rn(hash[i]);
  RC_CUDA(cudaMemcpy(n->hash_half, hh.data(), hh.size() * 2, cudaMemcpyHostToDevice), "cache upload");
  RC_CUDA(cudaMemset(n->mlp_m, 0, kNrcParams * 4), "cache init");
  RC_CUDA(cudaMemset(n->mlp_v, 0, kNrcParams * 4), "cache init");
  RC_CUDA(cudaMemset(n->mlp_g, 0, kNrcParams * 4), "cache init");
  RC_CUDA(cudaMemset(n->hash_m, 0, n->hash_n * 4), "cache init");
  RC_CUDA(cudaMemset(n->hash_v, 0, n->hash_n * 4), "cache init");
  RC_CUDA(cudaMemset(n->hash_g, 0, n->hash_n * 4), "cache init");
  launch_pack(n, 0);
  RC_CUDA(cudaGetLastError(), "cache pack");
  RC_CUDA(cudaDeviceSynchronize(), "cache init");
  n->steps = 0;
  return RC_OK;
}

}  // namespace

bool nrc_active(const rc_context* c) { return c && c->nrc; }
int nrc_first_level(const rc_context* c) { return c->nrc ? c->nrc->first : c->nlev; }
bool nrc_walks_near(const rc_context* c) { return c->nrc && c->nrc->ftab && c->qtab; }

cudaError_t nrc_check_read(unsigned long long* first, unsigned* count) {
#ifdef RC_CHECKED
  return check_read(first, count);
#else
  *first = 0;
  *count = 0;
  return cudaSuccess;
#endif
}

void nrc_release(rc_context* c) {
  if (!c || !c->nrc) return;
  free_state(c->nrc);
  c->nrc = nullptr;
}

// One solve's far cascades, all on the stream with no host wait:
//   1. walk this solve's training and held-out directions of every far probe
//      (the far levels' own walk queue), and read their targets;
//   2. refit (Adam) on the training samples;
//   3. held-out error of the refitted network per fallback tile -> flags ->
//      per level the serve decision (a level with at least
//      plain_level_fraction of its probes in flagged tiles runs on its walks);
//   4. walk what is still needed: the other directions of every word of a
//      level on its walks and of the words holding a probe of a flagged tile;
//   5. inference of the served probes with the network just scored, then per
//      level, top down, the merge from the network or from the walk records.
// Inference grid: one resident wave at most, kFwdGroups tiles per block at a time.
unsigned fwd_grid(const NrcState* n, int64_t ntiles) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((ntiles + kFwdGroups - 1) / kFwdGroups, n->fwd_blocks));
}

namespace {

// Walk of the far levels' queue.  Mode 0: the training and held-out
// directions (phase pair ph, ph + nph/2) of every word.  Mode 1: every other
// direction of the words k_nrc_words switches on, and every walk of the near
// levels that use the walk queue (nrc_walks_near).  The items of a far level
// are its selected directions x its slots, so skipped walks cost no lanes.
void far_walk(const rc_context* c, NrcState* n, cudaStream_t s, int mode, int ph) {
  QueueArgs q = n->fq;
  const int pair = ph % (n->nph / 2);
  int64_t items = 0;
  for (int k = 0; k < q.n; ++k) {
    QueueLevel& L = q.lv[k];
    const int i = L.level;
    const int64_t st = n->pair_start[i][pair], len = n->pair_len[i][pair];
    L.dsel_start = (int32_t)(mode == 0 ? st : (st + len) % L.dsel_len);
    L.dsel_n = (int32_t)(mode == 0 ? len : L.dsel_len - len);
    if (mode == 0) L.word_on = nullptr;
    L.item_begin = items;
    items += (int64_t)L.dsel_n * L.slots;
  }
  if (mode == 1 && nrc_walks_near(c))
    for (int k = 0; k < c->qargs.n; ++k) {
      const QueueLevel& nl = c->qargs.lv[k];
      if (nl.level >= n->first) continue;
      QueueLevel& L = q.lv[q.n++];
      L = nl;
      L.item_begin = items;
      items += (int64_t)L.slots * c->geom[L.level].ndirs;
    }
  q.total = items;
  if (!items) return;
  if (mode == 1) k_nrc_words<<<blocks_for(n->words.slot0[n->words.nlev], 128), 128, 0, s>>>(n->words);
  cudaMemsetAsync(n->fcounter, 0, sizeof(unsigned long long), s);
  if (n->ftab) {
    launch_table_walk(q, n->fq_resident, s);
  } else {
    const unsigned blocks = (unsigned)std::max<int64_t>(
        1, std::min<int64_t>((items + kQueueThreads - 1) / kQueueThreads, (int64_t)n->fq_resident));
    k_walk_queue<<<blocks, kQueueThreads, 0, s>>>(q);
  }
}

template <typename T>
void launch_heldout(const rc_context* c, NrcState* n, const NrcArgs& a, int64_t nho, const float* tho,
                    cudaStream_t s) {
  NrcLevelArgs la;
  memset(&la, 0, sizeof la);
  for (int i = 0; i < c->nlev; ++i) la.lv[i] = c->args[i];
  k_nrc_heldout<T><<<(unsigned)nho, kNrcThreads, 0, s>>>(a, la, n->pred, tho, n->tnum, n->tden);
}

template <typename T>
void launch_merge(const rc_context* c, const NrcState* n, int i, cudaStream_t s) {
  const LevelArgs& a = c->args[i];
  dim3 grid(blocks_for(a.P, 128), (unsigned)((a.n / 2) * (a.n / 2) / 2));
  if (i == c->nlev - 1) k_level_merge_nrc<T, true><<<grid, 128, 0, s>>>(a, n->base, i);
  else k_level_merge_nrc<T, false><<<grid, 128, 0, s>>>(a, n->base, i);
}

}  // namespace

rc_status nrc_enqueue_far(rc_context* c, cudaStream_t s) {
  RC_CUDA(check_prepare(), "checked build: range upload");
  NrcState* n = c->nrc;
  const int ph = (int)(n->solves % n->nph), hp = (ph + n->nph / 2) % n->nph;
  const int64_t tr0 = n->tile_begin[ph], ntr = n->tile_begin[ph + 1] - tr0;
  const int64_t ho0 = n->tile_begin[hp], nho = n->tile_begin[hp + 1] - ho0;
  float* ttr = n->target;
  float* tho = n->target + ntr * kNrcThreads * 4;
  // 1. the sample directions and their targets
  far_walk(c, n, s, 0, ph);
  NrcArgs a = n->base;
  if (ntr) {
    a.tiles = n->tiles + tr0;
    k_nrc_targets<<<blocks_for(ntr * kNrcThreads, 256), 256, 0, s>>>(a, c->vol, ntr, ttr);
  }
  if (nho) {
    a.tiles = n->tiles + ho0;
    k_nrc_targets<<<blocks_for(nho * kNrcThreads, 256), 256, 0, s>>>(a, c->vol, nho, tho);
  }
  // 2. refit on the training samples
  const int steps = std::max(1, n->prm.steps_per_solve);
  if (ntr) {
    RC_CUDA(cudaMemsetAsync(n->loss, 0, sizeof(float), s), "cache loss reset");
    n->loss_rows = 0;
    for (int st = 0; st < steps; ++st) {
      const int64_t a0 = ntr * st / steps, a1 = ntr * (st + 1) / steps;
      if (a1 <= a0) continue;
      int64_t rows = 0;
      for (int64_t t = a0; t < a1; ++t) rows += n->h_tiles[tr0 + t].n;
      n->loss_rows += rows;
      NrcArgs ta = n->base;
      ta.tiles = n->tiles + tr0 + a0;
      ta.ntiles = a1 - a0;
      ta.target = ttr + a0 * kNrcThreads * 4;
      ta.grad = n->mlp_g;
      ta.epos_grad = nullptr;
      ta.loss = n->loss;
      ta.inv_batch = 1.f / (float)std::max<int64_t>(rows, 1);
      k_nrc_train<<<(unsigned)std::min<int64_t>(a1 - a0, n->train_blocks), kNrcThreads, kTrainSmem, s>>>(ta);
      ++n->steps;
      launch_adam(n->mlp, n->mlp_g, n->mlp_m, n->mlp_v, nullptr, kNrcParams, n->prm, n->steps, false, s);
      launch_adam(n->hash_master, n->hash_g, n->hash_m, n->hash_v, n->hash_half, n->hash_n, n->prm, n->steps, true,
                  s);
      launch_pack(n, s);
    }
    RC_CUDA(cudaMemcpyAsync(n->h_loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, s), "cache loss");
  }
  // 3. held-out error of the refitted network -> flags -> serve decisions
  if (nho) {
    a.ntiles = nho;
    a.out = n->pred;
    k_nrc_forward<false><<<fwd_grid(n, nho), kFwdThreads, kFwdSmem, s>>>(a, nho);
    if (c->elem == 2) launch_heldout<__half>(c, n, a, nho, tho, s);
    else launch_heldout<float>(c, n, a, nho, tho, s);
    const float thr = n->prm.fallback_threshold;
    const int64_t cells = (int64_t)n->TX * n->TY * n->TZ;
    k_nrc_flags<<<blocks_for(cells, 256), 256, 0, s>>>(n->tnum, n->tden, n->tring, n->nph, ph, n->flag, cells,
                                                       thr * thr);
  }
  k_nrc_count<<<blocks_for(n->total_probes, 256), 256, 0, s>>>(n->base, n->flag, n->tile_shift, n->TX, n->TY,
                                                                n->total_probes, n->count);
  k_nrc_decide<<<1, kMaxCascades, 0, s>>>(n->base, n->count, n->plain, n->served_solves,
                                          n->prm.plain_level_fraction);
  // 4. the walks still needed
  far_walk(c, n, s, 1, ph);
  // 5. inference of the served probes with the network just scored, merges
  // top down
  k_nrc_forward<true><<<fwd_grid(n, n->enum_tiles), kFwdThreads, kFwdSmem, s>>>(n->base, n->enum_tiles);
  for (int i = c->nlev - 1; i >= n->first; --i) {
    if (c->elem == 2) launch_merge<__half>(c, n, i, s);
    else launch_merge<float>(c, n, i, s);
  }
  RC_CUDA(cudaGetLastError(), "cache launch");
  ++n->solves;
  return RC_OK;
}

}  // namespace rcx

using namespace rcx;

extern "C" {

int32_t rc_nrc_param_count(void) { return kNrcParams; }

rc_status rc_nrc_params_default(rc_nrc_params* out) {
  if (!out) {
    set_error("rc_nrc_params_default: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  memset(out, 0, sizeof *out);
  out->first_level = 2;
  out->hash_log2_entries = 19;
  out->base_resolution = 16;
  out->max_resolution = 512;
  out->learning_rate = 1e-2f;
  out->beta1 = 0.9f;
  out->beta2 = 0.99f;
  out->epsilon = 1e-10f;
  out->train_fraction_log2 = 4;
  out->steps_per_solve = 1;
  out->fallback_threshold = 0.01f;
  out->fallback_tile = 8;
  out->radiance_scale = 0.25f;
  out->plain_level_fraction = 0.5f;
  out->seed = 0x5EEDull;
  return RC_OK;
}

rc_status rc_nrc_enable(rc_context* c, const rc_nrc_params* prm) {
  if (check(c, "rc_nrc_enable", false) != RC_OK) return RC_ERR_INVALID_ARG;
  if (!prm) {
    set_error("rc_nrc_enable: params is NULL");
    return RC_ERR_INVALID_ARG;
  }
  const rc_nrc_params& q = *prm;
  const bool pow2_tile = q.fallback_tile >= 1 && (q.fallback_tile & (q.fallback_tile - 1)) == 0;
  if (q.first_level < 1 || q.first_level >= c->nlev || q.hash_log2_entries < 10 || q.hash_log2_entries > 24 ||
      q.base_resolution < 2 || q.max_resolution < q.base_resolution || q.max_resolution > 4096 ||
      !(q.learning_rate > 0.f) || !(q.beta1 >= 0.f && q.beta1 < 1.f) || !(q.beta2 >= 0.f && q.beta2 < 1.f) ||
      !(q.epsilon > 0.f) || q.train_fraction_log2 < 1 || q.train_fraction_log2 > 8 || q.steps_per_solve < 1 ||
      q.steps_per_solve > 64 || !(q.fallback_threshold >= 0.f) || !pow2_tile || !(q.radiance_scale > 0.f) ||
      !(q.plain_level_fraction >= 0.f && q.plain_level_fraction <= 1.f)) {
    set_error("rc_nrc_enable: invalid rc_nrc_params (first_level must be in [1, num_cascades))");
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_nrc_enable");
  nrc_release(c);
  NrcState* n = new NrcState();
  n->prm = q;
  n->first = q.first_level;
  n->nlev = c->nlev;
  n->nph = 1 << q.train_fraction_log2;
  n->T = (int64_t)1 << q.hash_log2_entries;
  n->hash_n = (int64_t)kNrcHashLevels * n->T * 2;
  auto fail = [&](rc_status st) {
    free_state(n);
    return st;
  };
  rc_status s;
  // hash grid
  NrcHash& hh = n->base.hash;
  hh.log2T = q.hash_log2_entries;
  const double bgrow = exp((log((double)q.max_resolution) - log((double)q.base_resolution)) / (kNrcHashLevels - 1));
  for (int l = 0; l < kNrcHashLevels; ++l) {
    hh.res[l] = std::max(1, (int)floor((double)q.base_resolution * pow(bgrow, (double)l) + 1e-9));
    hh.dres[l] = std::max(1, (int)floor(2.0 * pow(64.0, (double)l / (kNrcHashLevels - 1)) + 1e-9));
  }
  hh.inv_extent = 1.f / (float)std::max(c->p.grid[0], std::max(c->p.grid[1], c->p.grid[2]));
  if ((s = dev_alloc((void**)&n->hash_master, n->hash_n * 4, "hash grid")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->hash_m, n->hash_n * 4, "hash grid moments")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->hash_v, n->hash_n * 4, "hash grid moments")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->hash_g, n->hash_n * 4, "hash grid gradient")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->hash_half, n->hash_n * 2, "hash grid FP16")) != RC_OK) return fail(s);
  hh.table = n->hash_half;
  hh.grad = n->hash_g;
  // MLP
  float** mb[] = {&n->mlp, &n->mlp_m, &n->mlp_v, &n->mlp_g, &n->dbg_g};
  for (float** b : mb)
    if ((s = dev_alloc((void**)b, kNrcParams * 4, "network parameters")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->img, kImgBytes, "network weight image")) != RC_OK) return fail(s);
  // far levels: direction features, (R, T)
  n->base.first = n->first;
  n->base.nlev = c->nlev;
  int64_t queries = 0, dirs = 0;
  for (int i = n->first; i < c->nlev; ++i) {
    if (c->geom[i].probes() * c->geom[i].ndirs >= ((int64_t)1 << 31)) {
      set_error("rc_nrc_enable: cascade %d has 2^31 or more (probe, direction) queries", i);
      return fail(RC_ERR_UNSUPPORTED);
    }
    queries += c->geom[i].probes() * c->geom[i].ndirs;
    dirs += c->geom[i].ndirs;
    n->total_probes += c->geom[i].probes();
  }
  if ((s = dev_alloc((void**)&n->denc, dirs * kNrcDirFeat * 2, "direction features")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->rt, queries * 4 * 2, "cached (R, T)")) != RC_OK) return fail(s);
  {
    std::vector<__nv_bfloat16> de((size_t)dirs * kNrcDirFeat);
    int64_t dO = 0, qo = 0, t0 = 0;
    for (int i = n->first; i < c->nlev; ++i) {
      const LevelGeom& gm = c->geom[i];
      NrcLevel& L = n->base.lv[i];
      L.denc = n->denc + dO * kNrcDirFeat;
      L.rt = n->rt + qo * 4;
      L.P = gm.probes();
      L.ndirs = gm.ndirs;
      L.n = gm.n;
      for (int a = 0; a < 3; ++a) L.M[a] = gm.M[a];
      L.spacing = gm.spacing;
      n->base.tile0[i] = t0;
      t0 += (gm.probes() * gm.ndirs + kNrcThreads - 1) / kNrcThreads;
      const double pi = 3.14159265358979323846;
      for (int d = 0; d < gm.ndirs; ++d) {
        const int tx = d % gm.n, ty = d / gm.n;
        const double u = (2.0 * tx + 1.0) / gm.n - 1.0, v = (2.0 * ty + 1.0) / gm.n - 1.0;
        const double f[10] = {u, v, sin(pi * u), cos(pi * u), sin(pi * v), cos(pi * v),
                              sin(2 * pi * u), cos(2 * pi * u), sin(2 * pi * v), cos(2 * pi * v)};
        __nv_bfloat16* row = de.data() + (dO + d) * kNrcDirFeat;
        for (int k = 0; k < 10; ++k) row[k] = __float2bfloat16_rn((float)f[k]);
        for (int k = 0; k < 6; ++k) row[10 + k] = __float2bfloat16_rn(k == std::min(i - n->first, 5) ? 1.f : 0.f);
      }
      dO += gm.ndirs;
      qo += gm.probes() * gm.ndirs;
    }
    n->base.tile0[c->nlev] = t0;
    n->enum_tiles = t0;
    RC_CUDA(cudaMemcpy(n->denc, de.data(), de.size() * 2, cudaMemcpyHostToDevice), "rc_nrc_enable: upload");
  }
  n->base.img = n->img;
  n->base.params = n->mlp;
  n->base.scale = q.radiance_scale;
  n->base.err = c->err;
  // Far levels' walk geometry (the decimated-opacity words of the bit-parallel
  // walk).
  int64_t slot_total = 0;
  for (int i = n->first; i < c->nlev; ++i) {
    const LevelArgs& la = c->args[i];
    if (!c->bits_level[i] || !la.mask) {
      set_error("rc_nrc_enable: cascade %d has no bit-parallel walk (the learned form walks its words)", i);
      return fail(RC_ERR_UNSUPPORTED);
    }
    NrcLevel& L = n->base.lv[i];
    L.slots = c->rec_slots[i];
    L.wpp = la.wpp;
    L.l2px = la.l2px;
    n->words.slot0[i] = slot_total;
    slot_total += L.slots;
  }
  n->words.slot0[c->nlev] = slot_total;
  // Sample tiles by phase: every far probe with the directions of the phase
  // (nrc_dir_phase), up to 128 per tile; a tile's slot is its probe's index.
  {
    // Per level the directions ordered by phase pair (q, q + nph/2): the
    // training and held-out directions of a solve are one contiguous run,
    // the rest of the level the run after it (cyclically).
    std::vector<int32_t> dlist;
    std::vector<std::vector<int64_t>> list_b(kMaxCascades, std::vector<int64_t>(n->nph, 0)),
        list_e(kMaxCascades, std::vector<int64_t>(n->nph, 0));
    for (int i = n->first; i < c->nlev; ++i) {
      n->pair_start[i].assign(n->nph / 2, 0);
      n->pair_len[i].assign(n->nph / 2, 0);
      n->dlist_base[i] = (int64_t)dlist.size();
      for (int q = 0; q < n->nph / 2; ++q)
        for (int ph : {q, q + n->nph / 2}) {
          list_b[i][ph] = (int64_t)dlist.size();
          for (int d = 0; d < c->geom[i].ndirs; ++d)
            if (nrc_dir_phase(d, c->geom[i].n, n->nph) == ph) dlist.push_back(d);
          list_e[i][ph] = (int64_t)dlist.size();
        }
      for (int q = 0; q < n->nph / 2; ++q) {
        n->pair_start[i][q] = list_b[i][q] - n->dlist_base[i];
        n->pair_len[i][q] = list_e[i][q + n->nph / 2] - list_b[i][q];
      }
    }
    if ((int64_t)dlist.size() >= ((int64_t)1 << 31)) {
      set_error("rc_nrc_enable: too many far directions");
      return fail(RC_ERR_UNSUPPORTED);
    }
    n->tile_begin.assign(n->nph + 1, 0);
    for (int ph = 0; ph < n->nph; ++ph) {
      n->tile_begin[ph] = (int64_t)n->h_tiles.size();
      int32_t k = 0;
      for (int i = n->first; i < c->nlev; ++i) {
        const int64_t l0 = list_b[i][ph], len = list_e[i][ph] - l0;
        if (len == 0) continue;
        const int64_t P = c->geom[i].probes();
        if (len >= kNrcThreads) {  // tiles of one probe, 128 of its directions each
          for (int64_t p = 0; p < P; ++p, ++k)
            for (int64_t r0 = 0; r0 < len; r0 += kNrcThreads)
              n->h_tiles.push_back(NrcTile{i, (int32_t)p, (int32_t)(l0 + r0),
                                           (int32_t)std::min<int64_t>(kNrcThreads, len - r0), k, kNrcThreads});
        } else {  // tiles of 128 / len probes, all of their directions
          const int64_t per = kNrcThreads / len;
          for (int64_t p = 0; p < P; p += per) {
            const int64_t np = std::min<int64_t>(per, P - p);
            n->h_tiles.push_back(NrcTile{i, (int32_t)p, (int32_t)l0, (int32_t)(np * len), k, (int32_t)len});
            k += (int32_t)np;
          }
        }
      }
    }
    n->tile_begin[n->nph] = (int64_t)n->h_tiles.size();
    for (int ph = 0; ph < n->nph; ++ph) {
      const int hp = (ph + n->nph / 2) % n->nph;
      const int64_t ta = n->tile_begin[ph + 1] - n->tile_begin[ph], tb = n->tile_begin[hp + 1] - n->tile_begin[hp];
      n->max_tiles2 = std::max(n->max_tiles2, ta + tb);
      n->max_held = std::max(n->max_held, tb);
    }
    if ((s = dev_alloc((void**)&n->tiles, std::max<size_t>(1, n->h_tiles.size()) * sizeof(NrcTile), "cache tiles")) !=
        RC_OK)
      return fail(s);
    if (!n->h_tiles.empty())
      RC_CUDA(cudaMemcpy(n->tiles, n->h_tiles.data(), n->h_tiles.size() * sizeof(NrcTile), cudaMemcpyHostToDevice),
              "rc_nrc_enable: upload");
    if ((s = dev_alloc((void**)&n->dlist, std::max<size_t>(1, dlist.size()) * sizeof(int32_t),
                       "cache sample directions")) != RC_OK)
      return fail(s);
    if (!dlist.empty())
      RC_CUDA(cudaMemcpy(n->dlist, dlist.data(), dlist.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
              "rc_nrc_enable: upload");
    n->base.dlist = n->dlist;
  }
  if ((s = dev_alloc((void**)&n->target, std::max<int64_t>(1, n->max_tiles2) * kNrcThreads * 16, "cache targets")) !=
      RC_OK)
    return fail(s);
  if ((s = dev_alloc((void**)&n->pred, std::max<int64_t>(1, n->max_held) * kNrcThreads * 16, "cache predictions")) !=
      RC_OK)
    return fail(s);
  if ((s = dev_alloc((void**)&n->epos_grad, kNrcPosFeat * 4, "feature gradient probe")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->loss, sizeof(float), "cache loss")) != RC_OK) return fail(s);
  RC_CUDA(cudaMallocHost((void**)&n->h_loss, sizeof(float)), "rc_nrc_enable: pinned");
  *n->h_loss = 0.f;
  if ((s = dev_alloc((void**)&n->count, kMaxCascades * sizeof(unsigned), "cache counts")) != RC_OK) return fail(s);
  RC_CUDA(cudaMemset(n->count, 0, kMaxCascades * sizeof(unsigned)), "rc_nrc_enable: memset");
  if ((s = dev_alloc((void**)&n->plain, kMaxCascades * sizeof(int32_t), "cache serve decisions")) != RC_OK)
    return fail(s);
  if ((s = dev_alloc((void**)&n->served_solves, kMaxCascades * sizeof(unsigned long long), "cache serve counts")) !=
      RC_OK)
    return fail(s);
  RC_CUDA(cudaMemset(n->served_solves, 0, kMaxCascades * sizeof(unsigned long long)), "rc_nrc_enable: memset");
  {
    const std::vector<int32_t> all_plain(kMaxCascades, 1);  // every tile starts on the walk
    RC_CUDA(cudaMemcpy(n->plain, all_plain.data(), kMaxCascades * sizeof(int32_t), cudaMemcpyHostToDevice),
            "rc_nrc_enable: upload");
  }
  // exact texel solid angles of the far levels
  {
    std::vector<float> om;
    std::vector<int64_t> at(kMaxCascades, 0);
    for (int i = n->first; i < c->nlev; ++i) {
      at[i] = (int64_t)om.size();
      std::vector<double> w((size_t)c->geom[i].ndirs);
      rc_solid_angles(c->geom[i].n, w.data());
      for (double x : w) om.push_back((float)x);
    }
    if ((s = dev_alloc((void**)&n->omega, om.size() * sizeof(float), "far solid angles")) != RC_OK) return fail(s);
    RC_CUDA(cudaMemcpy(n->omega, om.data(), om.size() * sizeof(float), cudaMemcpyHostToDevice),
            "rc_nrc_enable: upload");
    for (int i = n->first; i < c->nlev; ++i) n->base.lv[i].omega = n->omega + at[i];
  }
  // the position and direction parts of every far query's hash
  {
    int64_t np = 0, nd = 0;
    for (int i = n->first; i < c->nlev; ++i) {
      np += c->geom[i].probes();
      nd += c->geom[i].ndirs;
    }
    if ((s = dev_alloc((void**)&n->hparts, (size_t)(np + nd) * kNrcHashLevels * sizeof(uint32_t),
                       "hash parts")) != RC_OK)
      return fail(s);
    RC_CUDA(check_prepare(), "checked build: range upload");
    int64_t po = 0, dof = np;
    for (int i = n->first; i < c->nlev; ++i) {
      NrcLevel& L = n->base.lv[i];
      L.hpos = n->hparts + po * kNrcHashLevels;
      L.hdir = n->hparts + dof * kNrcHashLevels;
      po += c->geom[i].probes();
      dof += c->geom[i].ndirs;
      const int64_t m = std::max<int64_t>(c->geom[i].probes(), c->geom[i].ndirs);
      k_nrc_hash_parts<<<blocks_for(m, 128), 128>>>(n->base, i);
    }
    RC_CUDA(cudaGetLastError(), "rc_nrc_enable: hash parts");
  }
  // fallback tiles: all start on the plain walk
  n->tile_shift = 0;
  while ((1 << n->tile_shift) < q.fallback_tile) ++n->tile_shift;
  n->TX = (c->p.grid[0] + q.fallback_tile - 1) / q.fallback_tile;
  n->TY = (c->p.grid[1] + q.fallback_tile - 1) / q.fallback_tile;
  n->TZ = (c->p.grid[2] + q.fallback_tile - 1) / q.fallback_tile;
  const int64_t cells = (int64_t)n->TX * n->TY * n->TZ;
  // per cell: this solve's held-out sums, and those of the last nph solves
  if ((s = dev_alloc((void**)&n->tnum, cells * 4, "tile errors")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->tden, cells * 4, "tile errors")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&n->tring, (size_t)n->nph * 2 * cells * 4, "tile error window")) != RC_OK) return fail(s);
  RC_CUDA(cudaMemset(n->tring, 0, (size_t)n->nph * 2 * cells * 4), "rc_nrc_enable: memset");
  if ((s = dev_alloc((void**)&n->flag, cells, "tile flags")) != RC_OK) return fail(s);
  RC_CUDA(cudaMemset(n->tnum, 0, cells * 4), "rc_nrc_enable: memset");
  RC_CUDA(cudaMemset(n->tden, 0, cells * 4), "rc_nrc_enable: memset");
  RC_CUDA(cudaMemset(n->flag, 1, cells), "rc_nrc_enable: memset");
  n->probe_tile.assign((size_t)cells, 0);
  for (int i = n->first; i < c->nlev; ++i) {
    const LevelGeom& gm = c->geom[i];
    const int h = gm.spacing >> 1;
    for (int z = 0; z < gm.M[2]; ++z)
      for (int y = 0; y < gm.M[1]; ++y)
        for (int x = 0; x < gm.M[0]; ++x)
          n->probe_tile[((size_t)((z * gm.spacing + h) >> n->tile_shift) * n->TY + ((y * gm.spacing + h) >> n->tile_shift)) *
                            n->TX +
                        ((x * gm.spacing + h) >> n->tile_shift)] = 1;
  }
  n->base.plain = n->plain;
  n->base.flag = n->flag;
  n->base.tile_shift = n->tile_shift;
  n->base.TX = n->TX;
  n->base.TY = n->TY;
  // The far levels' own walk queue: records of every far level, step tables
  // where every far level has one (else the walk's own DDA), and one switch
  // per word that the schedule sets before each walk.
  {
    if ((s = dev_alloc((void**)&n->word_on, std::max<int64_t>(1, slot_total), "far walk switches")) != RC_OK)
      return fail(s);
    RC_CUDA(cudaMemset(n->word_on, 0, std::max<int64_t>(1, slot_total)), "rc_nrc_enable: memset");
    size_t rec_words = 0;
    for (int i = n->first; i < c->nlev; ++i) rec_words += (size_t)c->geom[i].ndirs * n->base.lv[i].slots * 32;
    if ((s = dev_alloc((void**)&n->frec, rec_words * sizeof(uint32_t), "far walk records")) != RC_OK) return fail(s);
    if ((s = dev_alloc((void**)&n->fcounter, sizeof(unsigned long long), "far walk counter")) != RC_OK)
      return fail(s);
    QueueArgs& fq = n->fq;
    memset(&fq, 0, sizeof fq);
    fq.counter = n->fcounter;
    for (int a3 = 0; a3 < 3; ++a3) fq.G[a3] = c->p.grid[a3];
    fq.W = c->W;
    std::vector<uint2> steps;
    std::vector<int32_t> begin;
    std::vector<size_t> boff;
    bool tab_ok = !(getenv("RC_WALK_TABLES") && strcmp(getenv("RC_WALK_TABLES"), "0") == 0);
    size_t roff = 0;
    int64_t items = 0;
    char msg[256];
    for (int i = c->nlev - 1; i >= n->first; --i) {  // longest intervals first
      const LevelArgs& la = c->args[i];
      const LevelGeom& gm = c->geom[i];
      NrcLevel& NL = n->base.lv[i];
      QueueLevel& L = fq.lv[fq.n++];
      L.mask = la.mask;
      L.dirs = la.dirs;
      L.rec = n->frec + roff;
      NL.rec = L.rec;
      roff += (size_t)gm.ndirs * NL.slots * 32;
      L.item_begin = items;
      items += (int64_t)gm.ndirs * NL.slots;
      L.slots = NL.slots;
      L.l2s = la.l2s;
      L.l2px = la.l2px;
      L.wpp = la.wpp;
      for (int ax = 0; ax < 3; ++ax) L.M[ax] = la.M[ax];
      L.rep = la.rep;
      L.test_start = 0;
      L.level = i;
      L.word_on = n->word_on + n->words.slot0[i];
      NL.word_on = n->word_on + n->words.slot0[i];
      L.dsel = n->dlist + n->dlist_base[i];
      L.dsel_len = gm.ndirs;
      if (tab_ok) {
        std::vector<DirInfo> tab((size_t)gm.ndirs);
        if (!build_dir_table(gm, c->p.grid, tab.data(), msg, sizeof msg)) return fail(RC_ERR_UNSUPPORTED);
        boff.push_back(begin.size());
        for (int d = 0; d < gm.ndirs && tab_ok; ++d) {
          begin.push_back((int32_t)steps.size());
          const int64_t cnt = walk_steps(gm, c->p.grid, tab[d], false, nullptr, 0);
          if (cnt < 0 || steps.size() + (size_t)cnt > (size_t)INT32_MAX / 2) {
            tab_ok = false;
            break;
          }
          const size_t at = steps.size();
          steps.resize(at + (size_t)cnt);
          walk_steps(gm, c->p.grid, tab[d], false, reinterpret_cast<WalkStep*>(steps.data() + at), cnt);
        }
        begin.push_back((int32_t)steps.size());
      }
    }
    fq.total = items;
    if (tab_ok && !steps.empty()) {
      if ((s = dev_alloc((void**)&n->fsteps, steps.size() * sizeof(uint2), "far walk step tables")) != RC_OK)
        return fail(s);
      if ((s = dev_alloc((void**)&n->fstep_begin, begin.size() * sizeof(int32_t), "far walk step tables")) != RC_OK)
        return fail(s);
      RC_CUDA(cudaMemcpy(n->fsteps, steps.data(), steps.size() * sizeof(uint2), cudaMemcpyHostToDevice),
              "rc_nrc_enable: upload");
      RC_CUDA(cudaMemcpy(n->fstep_begin, begin.data(), begin.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
              "rc_nrc_enable: upload");
      for (int k = 0; k < fq.n; ++k) {
        fq.lv[k].steps = n->fsteps;
        fq.lv[k].step_begin = n->fstep_begin + boff[(size_t)k];
      }
      n->ftab = true;
    }
    int per_sm = 0, sms0 = 0;
    cudaDeviceGetAttribute(&sms0, cudaDevAttrMultiProcessorCount, c->device);
    if ((n->ftab ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_queue_tab, kQueueThreads, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_queue, kQueueThreads, 0)) !=
        cudaSuccess) {
      (void)cudaGetLastError();
      per_sm = 2;
    }
    n->fq_resident = std::max(1, sms0 * per_sm);
    NrcWordArgs& w = n->words;
    for (int i = 0; i < kMaxCascades; ++i) w.lv[i] = n->base.lv[i];
    w.first = n->first;
    w.nlev = c->nlev;
    w.plain = n->plain;
    w.flag = n->flag;
    w.tile_shift = n->tile_shift;
    w.TX = n->TX;
    w.TY = n->TY;
  }
  // kernels: shared memory and resident blocks
  RC_CUDA(cudaFuncSetAttribute(k_nrc_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem),
          "rc_nrc_enable: attribute");
  RC_CUDA(cudaFuncSetAttribute(k_nrc_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem),
          "rc_nrc_enable: attribute");
  RC_CUDA(cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem),
          "rc_nrc_enable: attribute");
  // Resident blocks: shared memory and registers per SM, and the tensor-memory
  // budget of 512 columns per SM (64 per inference warpgroup, 512 per training
  // block) -- so that no allocation ever waits.
  int sms = 0, smem_sm = 0, regs_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, c->device);
  cudaFuncAttributes fa{};
  int fwd_regs = 128;
  if (cudaFuncGetAttributes(&fa, k_nrc_forward<true>) == cudaSuccess) fwd_regs = std::max(fa.numRegs, 1);
  (void)cudaGetLastError();
  const int by_smem = smem_sm / (kFwdSmem + 1024);
  const int by_regs = regs_sm / (((fwd_regs + 7) & ~7) * kFwdThreads);
  const int by_tmem = 512 / (64 * kFwdGroups);
  n->fwd_blocks = std::max(1, sms * std::max(1, std::min(std::min(by_smem, by_regs), by_tmem)));
  n->train_blocks = std::max(1, sms);
  {
    std::vector<float> mlp, hash;
    init_params(n, mlp, hash);
    if ((s = upload_params(n, mlp, hash)) != RC_OK) return fail(s);
  }
  c->nrc = n;
  return RC_OK;
}

rc_status rc_nrc_disable(rc_context* c) {
  if (check(c, "rc_nrc_disable", false) != RC_OK) return RC_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_nrc_disable");
  nrc_release(c);
  return RC_OK;
}

namespace {
struct SaveHeader {
  uint32_t magic;    // 'RCNC'
  uint32_t version;  // 1
  uint32_t mlp_count;
  uint32_t pad;
  uint64_t hash_count;
  rc_nrc_params params;
};
constexpr uint32_t kSaveMagic = 0x434E4352u;
}  // namespace

rc_status rc_nrc_save(rc_context* c, void* out, int64_t bytes, int64_t* needed) {
  if (check(c, "rc_nrc_save", true) != RC_OK) return c ? RC_ERR_STATE : RC_ERR_INVALID_ARG;
  NrcState* n = c->nrc;
  const int64_t need = (int64_t)sizeof(SaveHeader) + (int64_t)kNrcParams * 4 + n->hash_n * 4;
  if (needed) *needed = need;
  if (!out) return RC_OK;
  if (bytes < need) {
    set_error("rc_nrc_save: need %lld bytes", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_nrc_save");
  SaveHeader h;
  memset(&h, 0, sizeof h);
  h.magic = kSaveMagic;
  h.version = 1;
  h.mlp_count = kNrcParams;
  h.hash_count = (uint64_t)n->hash_n;
  h.params = n->prm;
  char* o = static_cast<char*>(out);
  memcpy(o, &h, sizeof h);
  RC_CUDA(cudaMemcpy(o + sizeof h, n->mlp, kNrcParams * 4, cudaMemcpyDeviceToHost), "rc_nrc_save");
  RC_CUDA(cudaMemcpy(o + sizeof h + kNrcParams * 4, n->hash_master, n->hash_n * 4, cudaMemcpyDeviceToHost),
          "rc_nrc_save");
  return RC_OK;
}

rc_status rc_nrc_load(rc_context* c, const void* in, int64_t bytes) {
  if (check(c, "rc_nrc_load", true) != RC_OK) return c ? RC_ERR_STATE : RC_ERR_INVALID_ARG;
  NrcState* n = c->nrc;
  const int64_t need = (int64_t)sizeof(SaveHeader) + (int64_t)kNrcParams * 4 + n->hash_n * 4;
  if (!in || bytes != need) {
    set_error("rc_nrc_load: expected %lld bytes", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  SaveHeader h;
  memcpy(&h, in, sizeof h);
  if (h.magic != kSaveMagic || h.version != 1 || h.mlp_count != (uint32_t)kNrcParams ||
      h.hash_count != (uint64_t)n->hash_n || h.params.hash_log2_entries != n->prm.hash_log2_entries ||
      h.params.base_resolution != n->prm.base_resolution || h.params.max_resolution != n->prm.max_resolution ||
      h.params.first_level != n->prm.first_level) {
    set_error("rc_nrc_load: the saved cache does not match this cache's parameters");
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_nrc_load");
  const char* p = static_cast<const char*>(in) + sizeof h;
  std::vector<float> mlp(kNrcParams), hash((size_t)n->hash_n);
  memcpy(mlp.data(), p, kNrcParams * 4);
  memcpy(hash.data(), p + kNrcParams * 4, n->hash_n * 4);
  return upload_params(n, mlp, hash);
}

rc_status rc_nrc_get_stats(rc_context* c, rc_nrc_stats* out) {
  if (check(c, "rc_nrc_get_stats", true) != RC_OK) return c ? RC_ERR_STATE : RC_ERR_INVALID_ARG;
  if (!out) {
    set_error("rc_nrc_get_stats: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  NrcState* n = c->nrc;
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_nrc_get_stats");
  const int64_t cells = (int64_t)n->TX * n->TY * n->TZ;
  std::vector<uint8_t> f((size_t)cells);
  RC_CUDA(cudaMemcpy(f.data(), n->flag, cells, cudaMemcpyDeviceToHost), "rc_nrc_get_stats");
  memset(out, 0, sizeof *out);
  out->solves = n->solves;
  out->steps = n->steps;
  out->last_loss = n->loss_rows ? *n->h_loss / (float)n->loss_rows : 0.f;
  for (int64_t t = 0; t < cells; ++t)
    if (n->probe_tile[(size_t)t]) {
      ++out->tiles;
      out->fallback_tiles += f[(size_t)t] ? 1 : 0;
    }
  int32_t plain[kMaxCascades] = {};
  RC_CUDA(cudaMemcpy(plain, n->plain, sizeof plain, cudaMemcpyDeviceToHost), "rc_nrc_get_stats");
  for (int i = n->first; i < c->nlev; ++i)
    if (n->solves && !plain[i]) out->served_levels |= 1 << i;
  unsigned long long served[kMaxCascades] = {};
  RC_CUDA(cudaMemcpy(served, n->served_solves, sizeof served, cudaMemcpyDeviceToHost), "rc_nrc_get_stats");
  for (int i = 0; i < kMaxCascades; ++i) out->served_solves[i] = (int64_t)served[i];
  return RC_OK;
}

rc_status rc_nrc_query(rc_context* c, int32_t level, const int32_t* probes, const int32_t* dirs, int64_t count,
                       float* out) {
  if (check(c, "rc_nrc_query", true) != RC_OK) return c ? RC_ERR_STATE : RC_ERR_INVALID_ARG;
  NrcState* n = c->nrc;
  if (level < n->first || level >= c->nlev || count < 0 || (count && (!probes || !dirs || !out))) {
    set_error("rc_nrc_query: level must be a far cascade and the arrays non-NULL");
    return RC_ERR_INVALID_ARG;
  }
  if (!count) return RC_OK;
  std::vector<NrcTile> t((size_t)count);
  for (int64_t i = 0; i < count; ++i) {
    if (probes[i] < 0 || probes[i] >= c->geom[level].probes() || dirs[i] < 0 || dirs[i] >= c->geom[level].ndirs) {
      set_error("rc_nrc_query: query %lld out of range", (long long)i);
      return RC_ERR_INVALID_ARG;
    }
    t[i] = NrcTile{level, probes[i], dirs[i], 1, -1, 0};
  }
  DeviceGuard g(c->device);
  rc_status s = ensure_query(n, count);
  if (s != RC_OK) return s;
  cudaStream_t st = c->stream;
  RC_CUDA(cudaMemcpyAsync(n->qtiles, t.data(), count * sizeof(NrcTile), cudaMemcpyHostToDevice, st), "rc_nrc_query");
  RC_CUDA(check_prepare(), "checked build: range upload");
  NrcArgs a = n->base;
  a.tiles = n->qtiles;
  a.ntiles = count;
  a.out = n->qout;
  k_nrc_forward<false><<<fwd_grid(n, count), kFwdThreads, kFwdSmem, st>>>(a, count);
  RC_CUDA(cudaGetLastError(), "rc_nrc_query: launch");
  std::vector<float> raw((size_t)count * kNrcThreads * 4);
  RC_CUDA(cudaMemcpyAsync(raw.data(), n->qout, raw.size() * 4, cudaMemcpyDeviceToHost, st), "rc_nrc_query");
  RC_CUDA(cudaStreamSynchronize(st), "rc_nrc_query");
  int flag = 0;
  RC_CUDA(cudaMemcpy(&flag, c->err, sizeof flag, cudaMemcpyDeviceToHost), "rc_nrc_query");
  if (flag) {
    cudaMemset(c->err, 0, sizeof(int));
    set_error("rc_nrc_query: a bounded device-side wait ran out");
    return RC_ERR_TIMEOUT;
  }
  for (int64_t i = 0; i < count; ++i) nrc_serve(raw.data() + i * kNrcThreads * 4, n->prm.radiance_scale, out + 4 * i);
  return RC_OK;
}

rc_status rc_nrc_tile_gradient(rc_context* c, int32_t level, int32_t probe, int32_t d0, int32_t count,
                               const float* targets, float* param_grad, float* pos_grad) {
  if (check(c, "rc_nrc_tile_gradient", true) != RC_OK) return c ? RC_ERR_STATE : RC_ERR_INVALID_ARG;
  NrcState* n = c->nrc;
  if (level < n->first || level >= c->nlev || probe < 0 || probe >= c->geom[level].probes() || d0 < 0 ||
      count < 1 || count > kNrcThreads || d0 + count > c->geom[level].ndirs || !targets || !param_grad ||
      !pos_grad) {
    set_error("rc_nrc_tile_gradient: arguments out of range");
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  rc_status s = ensure_query(n, 1);
  if (s != RC_OK) return s;
  cudaStream_t st = c->stream;
  const NrcTile t{level, probe, d0, count, 0, 0};
  std::vector<float> tg((size_t)kNrcThreads * 4, 0.f);
  memcpy(tg.data(), targets, (size_t)count * 16);
  RC_CUDA(cudaMemcpyAsync(n->qtiles, &t, sizeof t, cudaMemcpyHostToDevice, st), "rc_nrc_tile_gradient");
  RC_CUDA(cudaMemcpyAsync(n->qout, tg.data(), tg.size() * 4, cudaMemcpyHostToDevice, st), "rc_nrc_tile_gradient");
  RC_CUDA(cudaMemsetAsync(n->dbg_g, 0, kNrcParams * 4, st), "rc_nrc_tile_gradient");
  RC_CUDA(cudaMemsetAsync(n->epos_grad, 0, kNrcPosFeat * 4, st), "rc_nrc_tile_gradient");
  RC_CUDA(check_prepare(), "checked build: range upload");
  NrcArgs a = n->base;
  a.hash.grad = nullptr;  // a probe: nothing is scattered into the table gradient
  a.tiles = n->qtiles;
  a.ntiles = 1;
  a.target = n->qout;
  a.grad = n->dbg_g;
  a.epos_grad = n->epos_grad;
  a.loss = nullptr;
  a.inv_batch = 1.f / (float)count;
  k_nrc_train<<<1, kNrcThreads, kTrainSmem, st>>>(a);
  RC_CUDA(cudaGetLastError(), "rc_nrc_tile_gradient: launch");
  RC_CUDA(cudaMemcpyAsync(param_grad, n->dbg_g, kNrcParams * 4, cudaMemcpyDeviceToHost, st), "rc_nrc_tile_gradient");
  RC_CUDA(cudaMemcpyAsync(pos_grad, n->epos_grad, kNrcPosFeat * 4, cudaMemcpyDeviceToHost, st),
          "rc_nrc_tile_gradient");
  RC_CUDA(cudaStreamSynchronize(st), "rc_nrc_tile_gradient");
  int flag = 0;
  RC_CUDA(cudaMemcpy(&flag, c->err, sizeof flag, cudaMemcpyDeviceToHost), "rc_nrc_tile_gradient");
  if (flag) {
    cudaMemset(c->err, 0, sizeof(int));
    set_error("rc_nrc_tile_gradient: a bounded device-side wait ran out");
    return RC_ERR_TIMEOUT;
  }
  return RC_OK;
}

}  // extern "C"
