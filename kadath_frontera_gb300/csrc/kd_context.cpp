#include "kd_context.hpp"

#include <cstring>
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
    ProfScope ps(this, PROF_LINE_PASS, flops);
    cuda_check(launch_line_passes(list, smem, dp, stream()), "line_passes kernel");
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
