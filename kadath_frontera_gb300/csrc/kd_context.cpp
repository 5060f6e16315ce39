#include "kd_context.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace kd {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::ostringstream os;
    os << what << ": " << cudaGetErrorName(e) << " (" << cudaGetErrorString(e) << ")";
    throw KdError(KD_ERR_CUDA, os.str());
  }
}

DeviceArena::~DeviceArena() {
  for (auto& c : chunks_) cudaFree(c.ptr);
}

void* DeviceArena::alloc_bytes(size_t n) {
  n = (n + 255) & ~size_t(255);
  if (n == 0) n = 256;
  while (true) {
    if (cur_chunk_ < chunks_.size()) {
      if (off_ + n <= chunks_[cur_chunk_].size) {
        void* p = chunks_[cur_chunk_].ptr + off_;
        off_ += n;
        return p;
      }
      cur_chunk_++;
      off_ = 0;
      continue;
    }
    size_t sz = n > chunk_ ? n : chunk_;
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, sz), "cudaMalloc(arena chunk)");
    chunks_.push_back({static_cast<char*>(p), sz});
  }
}

double* DeviceArena::alloc_doubles(size_t n) {
  return static_cast<double*>(alloc_bytes(n * sizeof(double)));
}

void DeviceArena::reset() {
  cur_chunk_ = 0;
  off_ = 0;
}

size_t DeviceArena::used() const {
  size_t u = 0;
  for (size_t i = 0; i < cur_chunk_ && i < chunks_.size(); i++) u += chunks_[i].size;
  return u + off_;
}

size_t DeviceArena::mark() const { return (cur_chunk_ << 40) | off_; }

void DeviceArena::release_to(size_t m) {
  cur_chunk_ = m >> 40;
  off_ = m & ((size_t(1) << 40) - 1);
}

Context::Context(int device) : device_(device) {
  cuda_check(cudaSetDevice(device), "cudaSetDevice");
  cuda_check(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, device), "SM count");
  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  cur_ = stream_;
  pool_cap_ = size_t(4) << 20;  // 4 Mi doubles = 32 MB of operator matrices
  cuda_check(cudaMalloc(&d_pool_, pool_cap_ * sizeof(double)), "cudaMalloc(matrix pool)");
  // a table of the autotuner for every context of the process (mode 1)
  if (const char* p = std::getenv("KD_TUNING_FILE"))
    if (*p) set_autotune(p, 1);
}

Context::~Context() {
  for (auto st : side_) cudaStreamSynchronize(st);
  cudaStreamSynchronize(stream_);
  for (auto st : side_) cudaStreamDestroy(st);
  for (auto e : side_ev_) cudaEventDestroy(e);
  if (fork_ev_) cudaEventDestroy(fork_ev_);
  for (auto& kv : itables_) cudaFree(kv.second);
  for (auto& kv : dtables_) cudaFree(kv.second);
  cudaFree(d_pool_);
  for (void* w : ws_) cudaFree(w);
  cudaStreamDestroy(stream_);
  // teardown reports nothing; its status must not surface as the "last
  // error" of this thread's next, unrelated launch check
  cudaGetLastError();
}

void* Context::workspace(int slot, size_t bytes, bool* fresh) {
  if (slot < 0 || slot >= WS_NSLOT) throw KdError(KD_ERR_ARG, "workspace slot out of range");
  if (fresh) *fresh = false;
  if (bytes > ws_cap_[slot]) {
    if (capturing) throw KdError(KD_ERR_STATE, "workspace grew during graph capture");
    cudaFree(ws_[slot]);  // synchronises the device: no launch still reads it
    ws_[slot] = nullptr;
    ws_cap_[slot] = 0;
    cuda_check(cudaMalloc(&ws_[slot], bytes), "cudaMalloc(workspace)");
    ws_cap_[slot] = bytes;
    if (fresh) *fresh = true;
  }
  return ws_[slot];
}

void Context::fork(int n) {
  if (n < 1) n = 1;
  if (!fork_ev_) cuda_check(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming), "cudaEventCreate");
  while (static_cast<int>(side_.size()) < n) {
    cudaStream_t st;
    cudaEvent_t e;
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate(side)");
    cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate(side)");
    side_.push_back(st);
    side_ev_.push_back(e);
  }
  cuda_check(cudaEventRecord(fork_ev_, stream_), "record fork");
  for (int i = 0; i < n; i++) cuda_check(cudaStreamWaitEvent(side_[i], fork_ev_, 0), "side waits main");
  nfork_ = n;
}

void Context::use(int i) { cur_ = (i < 0 || nfork_ == 0) ? stream_ : side_[i % nfork_]; }

void Context::join() {
  for (int i = 0; i < nfork_; i++) {
    cuda_check(cudaEventRecord(side_ev_[i], side_[i]), "record join");
    cuda_check(cudaStreamWaitEvent(stream_, side_ev_[i], 0), "main waits side");
  }
  nfork_ = 0;
  cur_ = stream_;
}

const double* Context::pool() {
  size_t n = bank_.pool_size();
  if (n > pool_uploaded_) {
    if (capturing) throw KdError(KD_ERR_STATE, "matrix pool grew during graph capture");
    if (n > pool_cap_) throw KdError(KD_ERR_ARG, "matrix pool capacity exceeded");
    cuda_check(cudaMemcpyAsync(d_pool_ + pool_uploaded_, bank_.pool().data() + pool_uploaded_,
                               (n - pool_uploaded_) * sizeof(double), cudaMemcpyHostToDevice, stream_),
               "upload matrix pool");
    cuda_check(cudaStreamSynchronize(stream_), "sync after pool upload");
    pool_uploaded_ = n;
  }
  return d_pool_;
}

const int* Context::table(const std::vector<int>& content) {
  auto it = itables_.find(content);
  if (it != itables_.end()) return it->second;
  if (capturing) throw KdError(KD_ERR_STATE, "new device table during graph capture");
  int* p = nullptr;
  size_t n = content.empty() ? 1 : content.size();
  cuda_check(cudaMalloc(&p, n * sizeof(int)), "cudaMalloc(table)");
  if (!content.empty()) {
    // ordered on this context's (non-blocking) stream and finished before
    // any later launch, whichever stream that launch goes to
    cuda_check(cudaMemcpyAsync(p, content.data(), content.size() * sizeof(int), cudaMemcpyHostToDevice, stream_),
               "upload table");
    cuda_check(cudaStreamSynchronize(stream_), "sync after table upload");
  }
  itables_[content] = p;
  return p;
}

const double* Context::dtable(const std::vector<double>& content) {
  auto it = dtables_.find(content);
  if (it != dtables_.end()) return it->second;
  if (capturing) throw KdError(KD_ERR_STATE, "new device table during graph capture");
  double* p = nullptr;
  size_t n = content.empty() ? 1 : content.size();
  cuda_check(cudaMalloc(&p, n * sizeof(double)), "cudaMalloc(dtable)");
  if (!content.empty()) {
    // ordered on this context's (non-blocking) stream and finished before
    // any later launch, whichever stream that launch goes to
    cuda_check(cudaMemcpyAsync(p, content.data(), content.size() * sizeof(double), cudaMemcpyHostToDevice, stream_),
               "upload dtable");
    cuda_check(cudaStreamSynchronize(stream_), "sync after dtable upload");
  }
  dtables_[content] = p;
  return p;
}

void Context::run_items(const std::vector<KdItem>& items, const std::vector<int>& batches) {
  const double* dp = pool();
  size_t i = 0;
  while (i < items.size()) {
    KdItemList list;
    std::memset(&list, 0, sizeof(list));
    int smem = 0;
    list.prefix[0] = 0;
    int n = 0;
    while (i < items.size() && n < KD_MAX_ITEMS) {
      const KdItem& it = items[i];
      list.items[n] = it;
      list.prefix[n + 1] = list.prefix[n] + batches[i];
      int d0 = it.n0, d1 = it.n1, d2 = it.n2;
      int m = d0 * d1 * d2;
      for (int q = 0; q < it.npass; q++) {
        if (it.pass[q].dim == 0) d0 = it.pass[q].n_out;
        if (it.pass[q].dim == 1) d1 = it.pass[q].n_out;
        if (it.pass[q].dim == 2) d2 = it.pass[q].n_out;
        if (d0 * d1 * d2 > m) m = d0 * d1 * d2;
      }
      if (m > smem) smem = m;
      n++;
      i++;
    }
    list.nitems = n;
    // algorithmic FP64 work: per pass, n_in multiply-adds per output value
    double flops = 0;
    for (int q = 0; q < n; q++) {
      const KdItem& it = list.items[q];
      int d0 = it.n0, d1 = it.n1, d2 = it.n2;
      double f = 0;
      for (int p = 0; p < it.npass; p++) {
        if (it.pass[p].dim == 0) d0 = it.pass[p].n_out;
        if (it.pass[p].dim == 1) d1 = it.pass[p].n_out;
        if (it.pass[p].dim == 2) d2 = it.pass[p].n_out;
        f += 2.0 * double(d0) * d1 * d2 * it.pass[p].n_in;
      }
      flops += f * (list.prefix[q + 1] - list.prefix[q]);
    }
    const LpShape sh = line_shape(list, smem, dp);
    ProfScope ps(this, PROF_LINE_PASS, flops);
    cuda_check(launch_line_passes(list, smem, dp, stream(), sh), "line_passes kernel");
    launches++;
  }
}

}  // namespace kd

namespace kd {

cudaEvent_t Context::next_event() {
  if (ev_next_ >= ev_pool_.size()) {
    cudaEvent_t e;
    cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    ev_pool_.push_back(e);
  }
  return ev_pool_[ev_next_++];
}

void Context::prof_enable(bool on) {
  prof_on_ = on;
  prof_.clear();
  prof_last_.clear();
  ev_next_ = 0;
}

// An event pair around a launch measures the time between the stream
// reaching the two events.  When the host issues launches more slowly than
// the GPU runs them, the stream drains and the pair would also count the
// wait for the host.  So whenever the last timed launch has already
// finished, a 200 us hold kernel (outside every pair) goes in first and the
// following launches queue behind it: the pairs then hold device time only.
void Context::prof_begin(int cat) {
  (void)cat;
  if (!prof_on_) return;
  cudaStream_t s = stream();
  cudaEvent_t last = nullptr;  // end event of the last timed launch on s
  for (auto& pe : prof_last_)
    if (pe.first == s) last = pe.second;
  bool drained = last == nullptr;
  if (!drained) {
    const cudaError_t q = cudaEventQuery(last);
    if (q == cudaErrorNotReady) {
      (void)cudaGetLastError();  // "not ready" is a status, not an error to keep
    } else {
      cuda_check(q, "cudaEventQuery (profile)");
      drained = true;
    }
  }
  if (drained) cuda_check(launch_hold(200000ull, s), "hold kernel (profile)");
  pending_begin_ = next_event();
  cuda_check(cudaEventRecord(pending_begin_, s), "cudaEventRecord");
}

void Context::prof_end(int cat, double work) {
  if (!prof_on_ || !pending_begin_) return;
  cudaEvent_t e = next_event();
  cuda_check(cudaEventRecord(e, stream()), "cudaEventRecord");
  prof_.push_back({cat, pending_begin_, e, work});
  bool found = false;
  for (auto& pe : prof_last_)
    if (pe.first == stream()) {
      pe.second = e;
      found = true;
    }
  if (!found) prof_last_.push_back({stream(), e});
  pending_begin_ = nullptr;
}

void Context::prof_read(double* ms, long long* count, double* work) {
  for (int c = 0; c < PROF_NCAT; c++) {
    ms[c] = 0;
    count[c] = 0;
    work[c] = 0;
  }
  cuda_check(cudaStreamSynchronize(stream_), "sync (profile)");
  for (auto& r : prof_) {
    float t = 0;
    cuda_check(cudaEventElapsedTime(&t, r.a, r.b), "cudaEventElapsedTime");
    ms[r.cat] += t;
    count[r.cat] += 1;
    work[r.cat] += r.work;
  }
}

}  // namespace kd

namespace kd {

// ------------------------------------------------------------ autotuner --
std::string LineTuner::key(const KdItemList& list, int smem_doubles) {
  const int nf = list.prefix[list.nitems];
  static const int fb[] = {1, 2, 4, 8, 16, 32, 64, 152, 512, 2048};
  int fhi = 0;
  for (int b : fb)
    if (nf <= b) {
      fhi = b;
      break;
    }
  int e = 64;
  while (e < smem_doubles) e *= 2;
  int np = 0;
  for (int i = 0; i < list.nitems; i++)
    if (list.items[i].npass > np) np = list.items[i].npass;
  std::ostringstream os;
  os << "f" << (fhi ? std::to_string(fhi) : std::string("big")) << "/e" << e << "/p" << np;
  return os.str();
}

// The table as written by save(): {"line_passes": {"<class>": {"cluster": c,
// "threads": t, "us": x}, ...}}.
void LineTuner::load(const std::string& p) {
  std::ifstream f(p);
  if (!f) return;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  size_t at = s.find("\"line_passes\"");
  if (at == std::string::npos) return;
  at = s.find('{', at);
  while (at != std::string::npos) {
    const size_t k0 = s.find('"', at + 1);
    if (k0 == std::string::npos) break;
    const size_t k1 = s.find('"', k0 + 1);
    const size_t b0 = s.find('{', k1);
    const size_t b1 = s.find('}', b0);
    if (k1 == std::string::npos || b0 == std::string::npos || b1 == std::string::npos) break;
    const std::string k = s.substr(k0 + 1, k1 - k0 - 1);
    const std::string body = s.substr(b0, b1 - b0 + 1);
    Entry en;
    auto num = [&](const char* name, double& out) {
      const size_t q = body.find(std::string("\"") + name + "\"");
      if (q == std::string::npos) return false;
      const size_t c = body.find(':', q);
      out = std::atof(body.c_str() + c + 1);
      return true;
    };
    double cl = 1, th = 128, us = 0;
    if (num("cluster", cl) && num("threads", th)) {
      num("us", us);
      en.shape.cluster = static_cast<int>(cl);
      en.shape.threads = static_cast<int>(th);
      en.us = us;
      table[k] = en;
    }
    at = s.find(',', b1);
    if (at == std::string::npos || s.find('"', at) == std::string::npos) break;
  }
}

void LineTuner::save() const {
  if (path.empty()) return;
  std::ofstream f(path);
  if (!f) return;
  f << "{\n  \"line_passes\": {";
  bool first = true;
  for (const auto& kv : table) {
    f << (first ? "\n" : ",\n") << "    \"" << kv.first << "\": {\"cluster\": " << kv.second.shape.cluster
      << ", \"threads\": " << kv.second.shape.threads << ", \"us\": " << kv.second.us << "}";
    first = false;
  }
  f << "\n  }\n}\n";
}

void Context::set_autotune(const std::string& path, int mode) {
  if (mode < 0 || mode > 2) throw KdError(KD_ERR_ARG, "autotune mode must be 0, 1 or 2");
  tuner.mode = mode;
  tuner.path = path;
  tuner.table.clear();
  if (mode > 0 && !path.empty()) tuner.load(path);
}

LpShape Context::line_shape(const KdItemList& list, int smem_doubles, const double* pool) {
  const int nf = list.prefix[list.nitems];
  if (tuner.mode == 0 || nf <= 0) return lp_default_shape(nf);
  const std::string k = LineTuner::key(list, smem_doubles);
  auto it = tuner.table.find(k);
  if (it != tuner.table.end()) {
    tuner.hits++;
    return it->second.shape;
  }
  if (tuner.mode < 2 || capturing || prof_on_) return lp_default_shape(nf);
  // Time every candidate shape on copies of the launch whose outputs go to
  // a scratch buffer (the real outputs may alias the inputs).
  KdItemList probe = list;
  size_t total = 0;
  std::vector<size_t> need(list.nitems);
  for (int i = 0; i < list.nitems; i++) {
    const KdItem& itm = list.items[i];
    int d0 = itm.n0, d1 = itm.n1, d2 = itm.n2;
    for (int q = 0; q < itm.npass; q++) {
      if (itm.pass[q].dim == 0) d0 = itm.pass[q].n_out;
      if (itm.pass[q].dim == 1) d1 = itm.pass[q].n_out;
      if (itm.pass[q].dim == 2) d2 = itm.pass[q].n_out;
    }
    const long long per = std::max<long long>(itm.out_stride, static_cast<long long>(d0) * d1 * d2);
    need[i] = static_cast<size_t>(list.prefix[i + 1] - list.prefix[i]) * static_cast<size_t>(per);
    total += need[i];
  }
  double* scratch = nullptr;
  cuda_check(cudaMalloc(&scratch, sizeof(double) * (total ? total : 1)), "cudaMalloc(autotune scratch)");
  size_t off = 0;
  for (int i = 0; i < list.nitems; i++) {
    probe.items[i].out = scratch + off;
    off += need[i];
  }
  std::vector<LpShape> cands;
  if (nf <= 64)
    for (int cl : {8, 4, 2}) cands.push_back({cl, 128});
  for (int th : {64, 128, 256}) cands.push_back({1, th});
  cudaStream_t s = stream();
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  LpShape best = lp_default_shape(nf);
  double best_us = 1e30;
  constexpr int reps = 5;
  for (const LpShape& c : cands) {
    cuda_check(launch_line_passes(probe, smem_doubles, pool, s, c), "autotune warm-up");
    cuda_check(cudaEventRecord(e0, s), "cudaEventRecord");
    for (int r = 0; r < reps; r++) cuda_check(launch_line_passes(probe, smem_doubles, pool, s, c), "autotune run");
    cuda_check(cudaEventRecord(e1, s), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(e1), "autotune sync");
    float ms = 0;
    cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    const double us = 1e3 * ms / reps;
    if (us < best_us) {
      best_us = us;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(scratch);
  tuner.table[k] = {best, best_us};
  tuner.tuned++;
  tuner.save();
  return best;
}

}  // namespace kd
