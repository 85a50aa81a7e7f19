// se2gpu_ensemble.cu -- batched ensemble of independent shots (see include/se2gpu.h).
//
// Every shot is an ordinary FP32 solver handle (se2gpu_create): its buffers,
// tensor maps and per-tile source/receiver lists are built exactly as for a
// single solve.  The ensemble groups the shots by polynomial degree and, per
// step, launches the batched persistent kernel once per group over a flattened
// (shot, tile) work list, so shots of any size share the GPU without per-shot
// launches.  The per-shot parameter tables live in device memory and depend
// only on which field buffer is the input and which staging slot the block
// uses; together with the step's index inside its block this makes the
// launches of a block of K steps identical on every repetition, so each block
// is captured once as a CUDA graph (per input buffer and slot) and replayed.
//
// Per block: the host gathers the block's STF values into pinned staging
// [shot][K][nsrc], one copy moves them to the device, the K steps run, one
// kernel per group samples the receivers of the block's last step, and one copy
// brings the receiver rows [shot][K][nrec][7] back; the host scatters them into
// the caller's arrays while the next block runs (two staging slots).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "se2gpu.h"
#include "se2gpu_internal.h"
#include "se2gpu_persist_launch.h"

namespace {

// a launch covers up to SE2P_BATCH_SHOTS consecutive shots of a group (their parameters
// are the kernel's parameter)
struct Chunk {
  int first = 0, nshots = 0;     // shots [first, first + nshots) of the group
  int item_off = 0, nitems = 0;  // its work list inside the group's
  int grid = 1;
};

struct Group {
  int p = 0, config = 0, nitems = 0;
  std::vector<int> shots;                  // ensemble shot indices, ascending
  std::vector<Chunk> chunks;
  se2p::Params *tab[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // [input buffer][slot], device
  std::vector<se2p::Params> htab[2][2];                                // the same, host (launch arguments)
  CUtensorMap *maps[2] = {nullptr, nullptr};                           // [input buffer], device [shot][4]
  int2 *items = nullptr;                                               // device (shot in its chunk, ty << 16 | tx)
};

}  // namespace

struct se2gpu_ensemble {
  int nshots = 0, precision = 0, block = 0, device = 0, nsm = 0, cur = 0;
  bool kahan = false, use_graphs = true;
  std::vector<se2gpu_solver *> sol;
  std::vector<int> nsrc, nrec, src_off, rec_off;   // per shot; offsets are prefix sums (nshots + 1)
  long total_nodes = 0;
  std::vector<Group> groups;
  double *stf_d[2] = {nullptr, nullptr}, *tr_d[2] = {nullptr, nullptr};   // device staging per slot
  double *stf_h[2] = {nullptr, nullptr}, *tr_h[2] = {nullptr, nullptr};   // pinned host staging
  cudaEvent_t ev_h2d[2] = {nullptr, nullptr}, ev_d2h[2] = {nullptr, nullptr};
  cudaStream_t stream = nullptr, own_stream = nullptr;
  cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // [input buffer][slot]
  int *err_dev = nullptr;
  long launches = 0, replays = 0;
  char err[512] = {0};
};

static thread_local char g_ens_create_err[512];

static int efail(se2gpu_ensemble *e, int code, const char *fmt, ...)
{
  char *buf = e ? e->err : g_ens_create_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, 512, fmt, ap);
  va_end(ap);
  return code;
}

#define ECK(e, call)                                                                                              \
  do {                                                                                                            \
    cudaError_t e_ = (call);                                                                                      \
    if (e_ != cudaSuccess) return efail((e), SE2GPU_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                                        __FILE__, __LINE__);                                                      \
  } while (0)

extern "C" const char *se2gpu_ensemble_last_error(const se2gpu_ensemble *e) { return e ? e->err : g_ens_create_err; }

static void drop_graphs(se2gpu_ensemble *e)
{
  for (int c = 0; c < 2; c++)
    for (int s = 0; s < 2; s++)
      if (e->graph[c][s]) {
        cudaGraphExecDestroy(e->graph[c][s]);
        e->graph[c][s] = nullptr;
      }
}

static void free_group(Group &g)
{
  for (int c = 0; c < 2; c++) {
    for (int s = 0; s < 2; s++) {
      cudaFree(g.tab[c][s]);
      g.tab[c][s] = nullptr;
      g.htab[c][s].clear();
    }
    cudaFree(g.maps[c]);
    g.maps[c] = nullptr;
  }
  cudaFree(g.items);
  g.items = nullptr;
  g.nitems = 0;
  g.chunks.clear();
}

extern "C" void se2gpu_ensemble_destroy(se2gpu_ensemble *e)
{
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  drop_graphs(e);
  for (Group &g : e->groups) free_group(g);
  for (int s = 0; s < 2; s++) {
    cudaFree(e->stf_d[s]); cudaFree(e->tr_d[s]);
    cudaFreeHost(e->stf_h[s]); cudaFreeHost(e->tr_h[s]);
    if (e->ev_h2d[s]) cudaEventDestroy(e->ev_h2d[s]);
    if (e->ev_d2h[s]) cudaEventDestroy(e->ev_d2h[s]);
  }
  cudaFree(e->err_dev);
  for (se2gpu_solver *h : e->sol) se2gpu_destroy(h);
  if (e->own_stream) cudaStreamDestroy(e->own_stream);
  delete e;
}

template <class T>
static int dput(se2gpu_ensemble *e, T **dst, const T *src, size_t n)
{
  *dst = nullptr;
  cudaError_t r = cudaMalloc((void **)dst, std::max<size_t>(n * sizeof(T), 16));
  if (r != cudaSuccess) {
    *dst = nullptr;
    cudaGetLastError();
    return efail(e, SE2GPU_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(r));
  }
  if (n) ECK(e, cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// (re)build a group's parameter tables, tensor-map tables and work list from
// its shots' handles (after creation and after a tile-configuration change)
static int build_group(se2gpu_ensemble *e, Group &g)
{
  free_group(g);
  const int K = e->block, ns = (int)g.shots.size();
  std::vector<se2p::Params> tab(ns);
  std::vector<CUtensorMap> maps(4 * (size_t)ns);
  std::vector<int2> items;
  for (int c = 0; c < 2; c++)
    for (int sl = 0; sl < 2; sl++) {
      for (int i = 0; i < ns; i++) {
        const int s = g.shots[i];
        se2gpu_solver *h = e->sol[s];
        se2p::Params prm = se2gpu_internal_f32_params(h);
        prm.u_out = h->pu[1 - c]; prm.w_out = h->pw[1 - c];
        prm.cu_out = h->pcu[1 - c]; prm.cw_out = h->pcw[1 - c];
        prm.a_out = h->pa;
        prm.stf = e->stf_d[sl] + (size_t)K * e->src_off[s];
        prm.rbuf_out = h->rbuf[0];   // written at even steps of a block
        prm.rbuf_in = h->rbuf[1];    // written at odd steps
        prm.trace_row = e->tr_d[sl] + (size_t)K * 7 * e->rec_off[s];
        prm.record = 0;
        prm.err = e->err_dev;
        tab[i] = prm;
      }
      int rc = dput(e, &g.tab[c][sl], tab.data(), tab.size());
      if (rc) return rc;
      g.htab[c][sl] = tab;
    }
  for (int c = 0; c < 2; c++) {
    for (int i = 0; i < ns; i++)
      for (int m = 0; m < 4; m++) maps[4 * (size_t)i + m] = e->sol[g.shots[i]]->maps[c][m];
    int rc = dput(e, &g.maps[c], maps.data(), maps.size());
    if (rc) return rc;
  }
  g.config = e->sol[g.shots[0]]->pconfig;
  const int occ = std::max(1, se2p::occupancy(g.p, g.config, e->kahan, true));
  for (int f = 0; f < ns; f += SE2P_BATCH_SHOTS) {
    Chunk ch;
    ch.first = f;
    ch.nshots = std::min(SE2P_BATCH_SHOTS, ns - f);
    ch.item_off = (int)items.size();
    for (int i = f; i < f + ch.nshots; i++) {
      se2gpu_solver *h = e->sol[g.shots[i]];
      if (h->pntx >= 32768 || h->pnty >= 32768) return efail(e, SE2GPU_ERR_ARG, "shot %d: more than 32767 tiles along an axis", g.shots[i]);
      for (int t = 0; t < h->pntx * h->pnty; t++) items.push_back(make_int2(i - f, ((t / h->pntx) << 16) | (t % h->pntx)));
    }
    ch.nitems = (int)items.size() - ch.item_off;
    ch.grid = std::max(1, std::min(ch.nitems, occ * e->nsm));
    g.chunks.push_back(ch);
  }
  g.nitems = (int)items.size();
  int rc = dput(e, &g.items, items.data(), items.size());
  if (rc) return rc;
  return 0;
}

extern "C" int se2gpu_ensemble_create(const se2gpu_problem *shots, int nshots, int precision, int block,
                                      se2gpu_ensemble **out)
{
  if (!out) return efail(nullptr, SE2GPU_ERR_ARG, "null output handle");
  *out = nullptr;
  if (!shots || nshots < 1) return efail(nullptr, SE2GPU_ERR_ARG, "at least one shot is required");
  if (precision != SE2GPU_FP32 && precision != SE2GPU_FP32_KAHAN)
    return efail(nullptr, SE2GPU_ERR_ARG, "the ensemble runs FP32 precisions only (33 or 32), not %d", precision);
  if (block < 1 || block > 4096) return efail(nullptr, SE2GPU_ERR_ARG, "block of %d steps outside 1..4096", block);
  se2gpu_ensemble *e = new se2gpu_ensemble();
  e->nshots = nshots; e->precision = precision; e->block = block;
  e->kahan = (precision == SE2GPU_FP32_KAHAN);
  int rc = 0;
#define TRY(x) do { if ((rc = (x)) != 0) { snprintf(g_ens_create_err, sizeof(g_ens_create_err), "%s", e->err); se2gpu_ensemble_destroy(e); return rc; } } while (0)
  if (cudaGetDevice(&e->device) != cudaSuccess) { cudaGetLastError(); delete e; return efail(nullptr, SE2GPU_ERR_CUDA, "no CUDA device"); }
  cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->device);
  if (cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete e;
    return efail(nullptr, SE2GPU_ERR_CUDA, "cudaStreamCreate failed");
  }
  e->stream = e->own_stream;
  e->src_off.assign(nshots + 1, 0);
  e->rec_off.assign(nshots + 1, 0);
  for (int s = 0; s < nshots; s++) {
    se2gpu_solver *h = nullptr;
    if (se2gpu_create(&shots[s], precision, 0, &h) != 0) {
      efail(e, SE2GPU_ERR_ARG, "shot %d: %s", s, se2gpu_create_error());
      TRY(SE2GPU_ERR_ARG);
    }
    e->sol.push_back(h);
    e->nsrc.push_back(h->nsrc);
    e->nrec.push_back(h->nrec);
    e->src_off[s + 1] = e->src_off[s] + h->nsrc;
    e->rec_off[s + 1] = e->rec_off[s] + h->nrec;
    e->total_nodes += h->nnodes;
  }
  for (int s = 0; s < nshots; s++) {
    const int p = e->sol[s]->p;
    auto it = std::find_if(e->groups.begin(), e->groups.end(), [p](const Group &g) { return g.p == p; });
    if (it == e->groups.end()) {
      e->groups.push_back(Group{});
      e->groups.back().p = p;
      it = e->groups.end() - 1;
    }
    it->shots.push_back(s);
  }
  std::sort(e->groups.begin(), e->groups.end(), [](const Group &a, const Group &b) { return a.p < b.p; });
  const int K = block;
  for (int sl = 0; sl < 2; sl++) {
    const size_t sb = std::max<size_t>((size_t)K * e->src_off[nshots] * 8, 16);
    const size_t tb = std::max<size_t>((size_t)K * 7 * e->rec_off[nshots] * 8, 16);
    if (cudaMalloc((void **)&e->stf_d[sl], sb) != cudaSuccess || cudaMalloc((void **)&e->tr_d[sl], tb) != cudaSuccess ||
        cudaMallocHost((void **)&e->stf_h[sl], sb) != cudaSuccess || cudaMallocHost((void **)&e->tr_h[sl], tb) != cudaSuccess) {
      cudaGetLastError();
      efail(e, SE2GPU_ERR_NOMEM, "staging buffers of %zu + %zu bytes", sb, tb);
      TRY(SE2GPU_ERR_NOMEM);
    }
    memset(e->stf_h[sl], 0, sb);
    if (cudaMemset(e->stf_d[sl], 0, sb) != cudaSuccess || cudaEventCreateWithFlags(&e->ev_h2d[sl], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_d2h[sl], cudaEventDisableTiming) != cudaSuccess) {
      efail(e, SE2GPU_ERR_CUDA, "staging set-up");
      TRY(SE2GPU_ERR_CUDA);
    }
  }
  if (cudaMalloc((void **)&e->err_dev, sizeof(int)) != cudaSuccess || cudaMemset(e->err_dev, 0, sizeof(int)) != cudaSuccess) {
    efail(e, SE2GPU_ERR_NOMEM, "error flag");
    TRY(SE2GPU_ERR_NOMEM);
  }
  for (se2gpu_solver *h : e->sol) h->stream = e->stream;
  for (Group &g : e->groups) {
    if (se2p::prepare(g.p, e->sol[g.shots[0]]->pconfig, e->kahan) != cudaSuccess) {
      efail(e, SE2GPU_ERR_CUDA, "batched kernel set-up for degree %d", g.p);
      TRY(SE2GPU_ERR_CUDA);
    }
    TRY(build_group(e, g));
  }
#undef TRY
  *out = e;
  return 0;
}

extern "C" int se2gpu_ensemble_set_stream(se2gpu_ensemble *e, void *stream)
{
  if (!e) return SE2GPU_ERR_ARG;
  ECK(e, cudaStreamSynchronize(e->stream));
  e->stream = stream ? (cudaStream_t)stream : e->own_stream;
  for (se2gpu_solver *h : e->sol) h->stream = e->stream;
  return 0;
}

extern "C" int se2gpu_ensemble_set_graphs(se2gpu_ensemble *e, int enable)
{
  if (!e) return SE2GPU_ERR_ARG;
  ECK(e, cudaStreamSynchronize(e->stream));
  e->use_graphs = enable != 0;
  if (!e->use_graphs) drop_graphs(e);
  return 0;
}

extern "C" int se2gpu_ensemble_set_tile_config(se2gpu_ensemble *e, int p, int config)
{
  if (!e) return SE2GPU_ERR_ARG;
  auto it = std::find_if(e->groups.begin(), e->groups.end(), [p](const Group &g) { return g.p == p; });
  if (it == e->groups.end()) return efail(e, SE2GPU_ERR_ARG, "no shot of degree %d", p);
  if (config < 0 || config >= se2p::num_configs(p)) return efail(e, SE2GPU_ERR_ARG, "no tile configuration %d for degree %d", config, p);
  ECK(e, cudaStreamSynchronize(e->stream));
  drop_graphs(e);
  for (int s : it->shots)
    if (se2gpu_set_tile_config(e->sol[s], config) != 0)
      return efail(e, SE2GPU_ERR_CUDA, "shot %d: %s", s, se2gpu_last_error(e->sol[s]));
  if (se2p::prepare(p, config, e->kahan) != cudaSuccess) return efail(e, SE2GPU_ERR_CUDA, "batched kernel set-up");
  return build_group(e, *it);
}

extern "C" int se2gpu_ensemble_tile_config(const se2gpu_ensemble *e, int p)
{
  if (!e) return SE2GPU_ERR_ARG;
  for (const Group &g : e->groups)
    if (g.p == p) return g.config;
  return SE2GPU_ERR_ARG;
}

// the launches of one block of n <= K steps starting from input buffer `cur`, slot sl
static int enqueue_block(se2gpu_ensemble *e, int cur, int sl, int n, cudaStream_t st)
{
  for (int k = 0; k < n; k++) {
    const int cin = cur ^ (k & 1);
    for (Group &g : e->groups)
      for (const Chunk &ch : g.chunks) {
        static thread_local se2p::BatchArgs ba;   // 28 KB: kept off the stack
        ba.maps = g.maps[cin] + 4 * (size_t)ch.first;
        ba.items = g.items + ch.item_off;
        ba.nshots = ch.nshots;
        ba.nitems = ch.nitems;
        ba.kblk = k;
        ba.write_a = (k == n - 1) ? 1 : 0;
        ba.err = e->err_dev;
        memcpy(ba.shots, g.htab[cin][sl].data() + ch.first, sizeof(se2p::Params) * ch.nshots);
        cudaError_t r = se2p::launch_batch(g.p, g.config, e->kahan, ba, ch.grid, st);
        if (r != cudaSuccess)
          return efail(e, SE2GPU_ERR_CUDA, "batched step kernel (degree %d): %s", g.p, cudaGetErrorString(r));
      }
  }
  for (Group &g : e->groups) {
    cudaError_t r = se2p::launch_record_batch(g.p, g.tab[cur][sl], (int)g.shots.size(), n - 1, st);
    if (r != cudaSuccess) return efail(e, SE2GPU_ERR_CUDA, "receiver kernel (degree %d): %s", g.p, cudaGetErrorString(r));
  }
  return 0;
}

static int launches_per_block(const se2gpu_ensemble *e, int n)
{
  int k = 0;
  for (const Group &g : e->groups) k += (int)g.chunks.size() * n + 1;
  return k;
}

static int run_block(se2gpu_ensemble *e, int sl, int n)
{
  const int cur = e->cur;
  if (e->use_graphs && n == e->block) {
    if (!e->graph[cur][sl]) {
      cudaGraph_t graph = nullptr;
      ECK(e, cudaStreamBeginCapture(e->own_stream, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue_block(e, cur, sl, n, e->own_stream);
      const cudaError_t ec = cudaStreamEndCapture(e->own_stream, &graph);
      if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
      ECK(e, ec);
      const cudaError_t ei = cudaGraphInstantiate(&e->graph[cur][sl], graph, 0);
      cudaGraphDestroy(graph);
      ECK(e, ei);
    }
    ECK(e, cudaGraphLaunch(e->graph[cur][sl], e->stream));
    e->replays++;
  } else {
    int rc = enqueue_block(e, cur, sl, n, e->stream);
    if (rc) return rc;
  }
  e->launches += launches_per_block(e, n);
  if (n & 1) {
    e->cur = 1 - cur;
    for (se2gpu_solver *h : e->sol) h->cur = e->cur;
  }
  return 0;
}

static int check_flag(se2gpu_ensemble *e)
{
  int flag = 0;
  ECK(e, cudaMemcpy(&flag, e->err_dev, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) return efail(e, SE2GPU_ERR_CUDA, "a batched step kernel gave up waiting for its tile copies (bounded wait expired)");
  return 0;
}

extern "C" int se2gpu_ensemble_advance(se2gpu_ensemble *e, int nsteps, const double *stf, double *traces)
{
  if (!e) return SE2GPU_ERR_ARG;
  if (nsteps < 0) return efail(e, SE2GPU_ERR_ARG, "negative step count");
  if (nsteps == 0) return 0;
  const int S = e->nshots, K = e->block;
  if (e->src_off[S] > 0 && !stf) return efail(e, SE2GPU_ERR_ARG, "stf values required for %d sources", e->src_off[S]);
  ECK(e, cudaSetDevice(e->device));
  const size_t sbytes = (size_t)K * e->src_off[S] * 8, tbytes = (size_t)K * 7 * e->rec_off[S] * 8;
  const bool want = traces && e->rec_off[S] > 0;
  int prev_n = 0, prev_k0 = 0, prev_sl = 0;
  auto scatter = [&](int sl, int k0, int n) {
    for (int s = 0; s < S; s++) {
      const size_t row = (size_t)7 * e->nrec[s];
      if (row)
        memcpy(traces + (size_t)7 * nsteps * e->rec_off[s] + (size_t)k0 * row, e->tr_h[sl] + (size_t)K * 7 * e->rec_off[s],
               (size_t)n * row * 8);
    }
  };
  int i = 0;
  for (int k0 = 0; k0 < nsteps; k0 += K, i++) {
    const int n = std::min(K, nsteps - k0), sl = i & 1;
    if (sbytes) {
      ECK(e, cudaEventSynchronize(e->ev_h2d[sl]));   // the slot's previous upload has left the pinned buffer
      for (int s = 0; s < S; s++)
        if (e->nsrc[s])
          memcpy(e->stf_h[sl] + (size_t)K * e->src_off[s], stf + (size_t)nsteps * e->src_off[s] + (size_t)k0 * e->nsrc[s],
                 (size_t)n * e->nsrc[s] * 8);
      ECK(e, cudaMemcpyAsync(e->stf_d[sl], e->stf_h[sl], sbytes, cudaMemcpyHostToDevice, e->stream));
      ECK(e, cudaEventRecord(e->ev_h2d[sl], e->stream));
    }
    int rc = run_block(e, sl, n);
    if (rc) return rc;
    if (want) {
      ECK(e, cudaMemcpyAsync(e->tr_h[sl], e->tr_d[sl], tbytes, cudaMemcpyDeviceToHost, e->stream));
      ECK(e, cudaEventRecord(e->ev_d2h[sl], e->stream));
      if (i > 0) {
        ECK(e, cudaEventSynchronize(e->ev_d2h[prev_sl]));
        scatter(prev_sl, prev_k0, prev_n);
      }
      prev_n = n; prev_k0 = k0; prev_sl = sl;
    }
  }
  ECK(e, cudaStreamSynchronize(e->stream));
  ECK(e, cudaGetLastError());
  if (want) scatter(prev_sl, prev_k0, prev_n);
  return check_flag(e);
}

extern "C" int se2gpu_ensemble_enqueue(se2gpu_ensemble *e, int nsteps)
{
  // device-resident variant for timing: replays blocks with the STF staging as
  // it stands and leaves the receiver rows on the device; no synchronisation
  if (!e) return SE2GPU_ERR_ARG;
  if (nsteps < 0) return efail(e, SE2GPU_ERR_ARG, "negative step count");
  ECK(e, cudaSetDevice(e->device));
  int i = 0;
  for (int k0 = 0; k0 < nsteps; k0 += e->block, i++) {
    int rc = run_block(e, 0, std::min(e->block, nsteps - k0));
    if (rc) return rc;
  }
  return 0;
}

extern "C" int se2gpu_ensemble_synchronize(se2gpu_ensemble *e)
{
  if (!e) return SE2GPU_ERR_ARG;
  ECK(e, cudaStreamSynchronize(e->stream));
  ECK(e, cudaGetLastError());
  return check_flag(e);
}

static int shot_arg(se2gpu_ensemble *e, int shot)
{
  if (!e) return SE2GPU_ERR_ARG;
  if (shot < 0 || shot >= e->nshots) return efail(e, SE2GPU_ERR_ARG, "shot %d outside 0..%d", shot, e->nshots - 1);
  return 0;
}

extern "C" int se2gpu_ensemble_get_fields(se2gpu_ensemble *e, int shot, double *u, double *v, double *a)
{
  int rc = shot_arg(e, shot);
  if (rc) return rc;
  ECK(e, cudaStreamSynchronize(e->stream));
  if ((rc = check_flag(e))) return rc;
  se2gpu_solver *h = e->sol[shot];
  h->cur = e->cur;
  if (se2gpu_get_fields(h, u, v, a) != 0) return efail(e, SE2GPU_ERR_CUDA, "shot %d: %s", shot, se2gpu_last_error(h));
  return 0;
}

extern "C" int se2gpu_ensemble_set_fields(se2gpu_ensemble *e, int shot, const double *u, const double *v, const double *a)
{
  int rc = shot_arg(e, shot);
  if (rc) return rc;
  ECK(e, cudaStreamSynchronize(e->stream));
  se2gpu_solver *h = e->sol[shot];
  h->cur = e->cur;
  if (se2gpu_set_fields(h, u, v, a) != 0) return efail(e, SE2GPU_ERR_CUDA, "shot %d: %s", shot, se2gpu_last_error(h));
  return 0;
}

extern "C" int se2gpu_ensemble_info(const se2gpu_ensemble *e, long *ints)
{
  if (!e || !ints) return SE2GPU_ERR_ARG;
  ints[0] = e->nshots;
  ints[1] = (long)e->groups.size();
  ints[2] = e->block;
  ints[3] = e->launches;
  ints[4] = e->replays;
  ints[5] = e->total_nodes;
  ints[6] = e->src_off[e->nshots];
  ints[7] = e->rec_off[e->nshots];
  long items = 0;
  for (const Group &g : e->groups) items += g.nitems;
  ints[8] = items;
  return 0;
}
