// Per-thread solver context: CUDA stream, FP64 matrix pool, device tables,
// bump arenas for field storage, and error state.  One context drives one
// GPU; the C ABI hands it out as an opaque kd_ctx*.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "kadath_gb300.h"  // status codes
#include "kd_bases.hpp"
#include "kd_device.hpp"

namespace kd {

struct KdError : std::runtime_error {
  int code;
  KdError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what);

// Bump allocator over large device chunks; reset() recycles everything.
// Allocation order is deterministic, so a replayed sequence of allocations
// returns the same addresses (needed for CUDA-graph replays).
class DeviceArena {
 public:
  explicit DeviceArena(size_t chunk_bytes = size_t(256) << 20) : chunk_(chunk_bytes) {}
  ~DeviceArena();
  double* alloc_doubles(size_t n);
  void* alloc_bytes(size_t n);
  void reset();
  size_t used() const;
  size_t mark() const;          // current position (for scoped reuse)
  void release_to(size_t mark);

 private:
  struct Chunk {
    char* ptr;
    size_t size;
  };
  std::vector<Chunk> chunks_;
  size_t cur_chunk_ = 0, off_ = 0, chunk_;
};

// Launch shapes of the line passes picked by timing (the project's
// autotuner): per shape class of a launch (fields, largest stage, passes)
// the fastest candidate shape, kept in a JSON table.
class LineTuner {
 public:
  int mode = 0;  // 0: default rule; 1: the table (default rule for classes it lacks); 2: also time the classes it lacks and save
  std::string path;
  struct Entry {
    LpShape shape;
    double us = 0;
  };
  std::map<std::string, Entry> table;
  long long tuned = 0, hits = 0;
  void load(const std::string& p);
  void save() const;
  static std::string key(const KdItemList& list, int smem_doubles);
};

class Context {
 public:
  explicit Context(int device);
  ~Context();

  int device() const { return device_; }
  // SMs the context's grid-wide kernels may spread over (the LU's sweeps,
  // matvecs, cooperative panels and trailing updates): all of the device's
  // unless a budget is set, so that contexts run side by side (concurrent
  // instances) share the GPU instead of taking turns.
  int sms() const { return (sm_budget_ > 0 && sm_budget_ < nsm_) ? sm_budget_ : nsm_; }
  // Limit of one grid-barrier wait in the solver's cooperative kernels (LU
  // panel, triangular sweeps); after it the kernel sets an error flag and
  // returns, and the call reports KD_ERR_TIMEOUT.
  unsigned long long grid_wait_ns = 2000000000ull;
  // Failure injection for tests of that path: nonzero raises every
  // grid-barrier target by one, so that no barrier completes and every wait
  // runs out after grid_wait_ns.
  int stall_waits = 0;
  void set_sm_budget(int n) { sm_budget_ = n; }
  // The stream work is issued on: the context's main stream, or one of the
  // side streams between fork() and join().
  cudaStream_t stream() const { return cur_; }
  cudaStream_t main_stream() const { return stream_; }
  // Side streams for independent work (the per-domain equations of a value
  // pass): fork() makes n side streams wait for the main stream's work so
  // far, use(i) issues on side stream i % n (i < 0: the main stream), join()
  // makes the main stream wait for every side stream and goes back to it.
  void fork(int n);
  void use(int i);
  void join();

  MatrixBank& bank() { return bank_; }
  // Makes sure every matrix in the bank is present in the device pool.
  const double* pool();
  // Device copy of an int table, cached by content.
  const int* table(const std::vector<int>& content);
  // Device copy of a double table, cached by content.
  const double* dtable(const std::vector<double>& content);

  // Arena every DVal operation allocates from.  Normally the per-pass
  // scratch arena; redirect_scratch() points it at another arena (the
  // system's cache of node values) and returns the previous one.
  DeviceArena& scratch() { return *active_scratch_; }
  DeviceArena* redirect_scratch(DeviceArena* a) {
    DeviceArena* old = active_scratch_;
    active_scratch_ = a ? a : &scratch_;
    return old;
  }
  DeviceArena& persistent() { return persistent_; }

  // Device workspaces owned by the context, one per slot, grown on demand
  // (contents are not kept across growth; *fresh tells the caller the
  // buffer is new).  Work of one context is ordered on its streams, so
  // contexts driven from different host threads never share a workspace.
  // WS_TC_A2 / WS_TC_B2: the packed operands of the update that runs as
  // 16-CTA clusters on a side stream, beside updates on the main stream
  enum WorkSlot : int { WS_TC_A = 0, WS_TC_B = 1, WS_TC_FLAG = 2, WS_TC_A2 = 3, WS_TC_B2 = 4, WS_NSLOT = 5 };
  void* workspace(int slot, size_t bytes, bool* fresh = nullptr);

  // While a CUDA graph is being captured no host->device upload may happen;
  // the first (uncaptured) evaluation fills every cache.
  bool capturing = false;

  std::string last_error;

  // Packs items into launches of at most KD_MAX_ITEMS and runs them.
  void run_items(const std::vector<KdItem>& items, const std::vector<int>& batches);

  // Statistic: number of kernels this context launched.
  long long launches = 0;

  // Optional per-category timing of launches (CUDA events on this stream)
  // with the algorithmic work (bytes or flops) each launch performs.
  enum ProfCat : int {
    PROF_LINE_PASS = 0,  // separable transforms / 1-D coefficient operators (work: FP64 flops)
    PROF_EW = 1,         // elementwise algebra at collocation points
    PROF_GATHER = 2,     // tau export / affecte_tau gathers
    PROF_LU_PANEL = 3,         // partial-pivoting panels (work: bytes, the panel read and written once)
    PROF_LU_SWAP_TRSM = 4,     // row exchanges and the U12 solve (work: bytes of A12 read and written)
    PROF_LU_GEMM = 5,          // trailing update (work: HBM bytes of the tensor-core update, flops of the FP64 GEMM)
    PROF_LU_SOLVE = 6,         // one triangular sweep (work: bytes of the triangle read)
    PROF_GMRES = 7,            // refinement matvecs and vector ops
    PROF_LU_PANEL_STATIC = 8,  // static-pivot panels (work: bytes, the panel read and written once)
    PROF_NCAT = 9,
  };
  // The autotuner of the line passes (see LineTuner); path "" keeps the
  // table in memory only.
  void set_autotune(const std::string& path, int mode);
  LineTuner tuner;
  // The shape for one line-pass launch: the table's, or the default rule; in
  // mode 2 an unknown class is timed first (never during a capture).
  LpShape line_shape(const KdItemList& list, int smem_doubles, const double* pool);
  void prof_enable(bool on);
  bool prof_on() const { return prof_on_; }
  void prof_begin(int cat);
  void prof_end(int cat, double work);
  // Sums elapsed ms, launch counts and work per category (synchronises).
  void prof_read(double* ms, long long* count, double* work);

 private:
  bool prof_on_ = false;
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_next_ = 0;
  struct ProfRec {
    int cat;
    cudaEvent_t a, b;
    double work;
  };
  std::vector<ProfRec> prof_;
  cudaEvent_t pending_begin_ = nullptr;
  std::vector<std::pair<cudaStream_t, cudaEvent_t>> prof_last_;
  cudaEvent_t next_event();

 public:

 private:
  int device_;
  int nsm_ = 0, sm_budget_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaStream_t cur_ = nullptr;
  std::vector<cudaStream_t> side_;
  std::vector<cudaEvent_t> side_ev_;
  cudaEvent_t fork_ev_ = nullptr;
  int nfork_ = 0;
  MatrixBank bank_;
  double* d_pool_ = nullptr;
  size_t pool_cap_ = 0, pool_uploaded_ = 0;
  std::map<std::vector<int>, int*> itables_;
  std::map<std::vector<double>, double*> dtables_;
  DeviceArena scratch_;
  DeviceArena* active_scratch_ = &scratch_;
  DeviceArena persistent_{size_t(64) << 20};
  void* ws_[WS_NSLOT] = {};
  size_t ws_cap_[WS_NSLOT] = {};
};

// Times one launch (or a short sequence) when profiling is on.
struct ProfScope {
  Context* c;
  int cat;
  double work;
  ProfScope(Context* ctx, int category, double w) : c(ctx), cat(category), work(w) { c->prof_begin(cat); }
  ~ProfScope() { c->prof_end(cat, work); }
};

// Builds the pass description of a 1-D operator along `dim` for a field of
// current dims `dims` whose per-line bases are given by the basis table of
// that dim.  Used by transforms and by coefficient-space operators.
struct LinePassSpec {
  int dim, n_in, n_out, mat_ld;
  std::vector<int> offsets;  // per line, -1 for zero lines
};

}  // namespace kd
