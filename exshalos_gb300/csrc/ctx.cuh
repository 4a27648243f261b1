// Library context: cached FFT plans, device work buffers and the results of
// the last halo call.  One context per host thread.
#pragma once
#include <functional>
#include <map>
#include <tuple>
#include <vector>
#include <string>

#include "exh_common.cuh"
#include "fft.cuh"

namespace exh {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return EXH_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + 256;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      exh_set_error_msg("device allocation failed", __FILE__, __LINE__);
      return EXH_E_NOMEM;
    }
    cap = want;
    return EXH_OK;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

struct HostTables {
  int Ncells = 0, Nr = 0;
  std::vector<float> Sig_grid, Btab;
  std::vector<double> M, Int;
};

// results of the last halo call (device pointers into the context buffers)
struct HaloState {
  int64_t nh = 0, np = 0, nproc = 0;
  int nd[3] = {0, 0, 0};
  size_t ng = 0;
  float *posh = nullptr, *velh = nullptr, *Mh = nullptr;
  int *count = nullptr, *xc = nullptr;
  float *delta = nullptr, *pos = nullptr, *vel = nullptr;
  int *flag = nullptr, *hid = nullptr;
  HostTables tab;
};

enum BufId {
  B_WORK = 0,     // complex work array of the FFTs
  B_WORK2,        // second complex work array
  B_DELTA,        // float field
  B_GRID,         // float grid
  B_PHI1,         // first-order potential (float)
  B_PHI2,         // second-order potential (float)
  B_S,            // displacements [3][ng]
  B_V,            // particle positions / velocities [ng][3]
  B_VEL,          // velocity planes [3][ng]
  B_CROSS,        // first-crossing map staging (u8 per cell)
  B_LADDER,       // Fourier modes kept for the smoothing ladder (float2[nk])
  B_LADDERW,      // ladder window table W(kR) per radius and |n|^2
  B_CICACC,       // CIC fixed-point accumulator (u64 per cell)
  B_FLAG,         // int32 halo flag per cell
  B_PEAKS,        // peak keys/ids (sort ping-pong)
  B_PEAKS2,
  B_SORT,         // sort scratch
  B_HALO,         // halo records
  B_HALO2,
  B_HALO3,        // growth hand-off lists
  B_POSH,         // halo positions / velocities
  B_MH,
  B_TAB,          // device copies of tables
  B_HODIN,        // galaxy population: staged halo inputs
  B_HOD,          // galaxy population: per-halo work, stream, tables
  B_HODG,         // galaxy population: the galaxies of the last call
  B_SCRATCH,      // per-block partials, counters
  B_GAUSS,        // taus field stream: deviates (or phases) in draw order
  B_TAUS,         // taus field stream: jump matrices, per-chunk counts and scans
  B_HSUM,         // halo sums: the larger halos handed to the warp pass
  B_HOSTIO,       // staging for host pointers
  B_HOSTIO2,
  B_COUNT
};

struct DiffState;     // differentiable forward kept for its adjoint (diff.cu)

struct Ctx {
  int device = 0;
  std::map<std::tuple<int, int, int>, FFTPlan3D> plans;
  DevBuf buf[B_COUNT];
  HaloState halos;
  int64_t launches = 0;
  int verbose = 0;     // progress lines on stdout, as the reference's verbose flag
  // host tables of the last distinct (P(k), cosmology, cell, barrier) input
  std::string tab_key;
  HostTables tab_cache;
  // device tables reused while their inputs repeat
  std::string amp_key;                  // field amplitudes (B_TAB)
  std::string taus_key;                 // taus field draws (B_GAUSS): box, seed, fixed
  const void* taus_jump_at = nullptr;   // B_TAUS address the jump matrices were copied to
  // accepted pairs of the last taus stream, copied to pinned host memory and
  // checked against the draws needed at the caller's next synchronisation
  unsigned* taus_have_host = nullptr;
  long long taus_need = 0;
  bool taus_pending = false;
  int shell_ncells = -1, shell_nmin = -1, shell_gmax = 0;   // shell offsets (B_HALO2)
  size_t shell_ncap = 0, shell_nall = 0;
  std::string mass_key;                 // mass-function splines (B_WORK2)
  std::string ladder_key;               // ladder window table (B_LADDERW)
  std::string ladder_tab_key;           // ladder radii and barriers (host)
  std::string ladder_seen_key, ladder_graph_key;
  cudaGraphExec_t ladder_graph = nullptr;   // captured radius loop
  // the halo finder's level loop (sort) and round loop (growth) as graphs
  // whose while node the kernels end on the device; rebuilt when their
  // arguments change
  cudaGraph_t sort_graph_src = nullptr;
  cudaGraphExec_t sort_graph = nullptr;
  std::string sort_graph_key;
  struct GraphEntry {
    std::string key;
    cudaGraph_t src = nullptr;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<GraphEntry> grow_graphs;
  cudaStream_t capture = nullptr;           // stream used only to capture graph bodies
  int capture_stream(cudaStream_t* out);
  std::vector<float> ladder_R, ladder_B;
  // sorted peaks of the last grid given to exh_find_halos (B_PEAKS2), by digest
  unsigned long long peak_hash = 0;
  int peak_nd[3] = {0, 0, 0};
  int64_t peak_np = 0;
  float* peak_key = nullptr;
  unsigned* peak_id = nullptr;
  DiffState* diff = nullptr;
  // second stream for work that runs beside the halo finder (LPT), created
  // on first use; fork/join events
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int side_stream(cudaStream_t* out);
  // the stream for work forked from st: the side stream, or st itself while
  // kernel-class timing is on (each class's event time then covers its own
  // kernels only, not the ones of the other stream running beside them)
  int fork_stream(cudaStream_t st, cudaStream_t* out);
  // galaxies of the last exh_hod_populate (B_HODG)
  int64_t hod_ng = -1;
  int hod_vel = 0;
  size_t hod_off = 0;                   // galaxies start after the random stream
  // lanes of the batched runner: contexts with their own streams
  std::vector<exh_ctx*> lane_ctx;
  std::vector<cudaStream_t> lane_st;
  int get_plan(int nx, int ny, int nz, FFTPlan3D** out);
};

void diff_state_release(Ctx& c);

// A graph of one while node.  `body` enqueues the loop body on the stream it
// is given (captured into the node's body graph); its kernels end the loop
// with cudaGraphSetConditional(handle, 0).  The condition is 1 at every
// launch, so the body runs at least once.
int build_while_graph(Ctx& c, const std::function<int(cudaStream_t, cudaGraphConditionalHandle)>& body,
                      cudaGraph_t* src_out, cudaGraphExec_t* exec_out);

}  // namespace exh

struct exh_ctx {
  exh::Ctx c;
};
