// Halo finder of src/exshalos/find_halos.c on the GPU.
#pragma once
#include "ctx.cuh"
#include "setup.h"

namespace exh {

// temporary per-cell labels while halos are grown (int32):
//   FREE               unclaimed
//   r >= 0             inside the sphere grown from processed peak r
//   -(r + 2)           centre cell of processed peak r
constexpr int FLAG_FREE = -1;

struct ShellTable {
  // offsets packed (i+128) | (j+128) << 8 | (k+128) << 16, ordered by
  // r^2 then i, j, k ascending (the loop order of find_halos.c:295-306)
  int* off_cap = nullptr;     // |component| <= nmin/2 (growth and shrink)
  int* start_cap = nullptr;   // [gmax + 2]
  int* off_all = nullptr;     // uncapped (flag writes, find_halos.c:343-354)
  int* start_all = nullptr;
  int gmax = 0;               // last shell in the tables
};

struct HaloDev {
  // peaks
  float* key = nullptr;       // sorted ascending (reference quicksort order)
  unsigned* id = nullptr;     // linear cell index of each peak
  int64_t np = 0;
  int64_t nproc = 0;          // peaks the reference loop visits
  // per processed peak r (processing order = descending sorted index)
  int* gfree = nullptr;       // exclusion-free first rejected shell
  int* gfin = nullptr;        // final grows_tmp (flag radius^2 bound)
  int* cnt = nullptr;         // member count (0: no halo)
  unsigned char* state = nullptr;  // 0 pending, 1 resolved
  int* hid = nullptr;         // halo index of r (kept) or -1
  // halos in output order
  int64_t nh = 0;
  int* hpeak = nullptr;       // processed-peak index of each halo
  int* flag = nullptr;        // per cell, temporary labels
  unsigned* resv = nullptr;   // per cell reservations
  unsigned* words = nullptr;  // per processed peak: 4-byte words the growth touched (timing only)
};

struct HaloScalars {
  float Bmin;
  float Mtot;
  int Ncells;
  int Nmin;
  int nmin_half;
  int n0, n1, n2;
};

int build_shell_tables(Ctx& c, const BoxParams& b, int Ncells, ShellTable* t, cudaStream_t st);
int find_peaks(Ctx& c, const float* delta, const BoxParams& b, HaloDev* h, cudaStream_t st);
int sort_peaks(Ctx& c, HaloDev* h, cudaStream_t st);
int grow_halos(Ctx& c, const float* delta, const BoxParams& b, const HaloScalars& hs, const float* Btab_dev,
               const ShellTable& t, HaloDev* h, cudaStream_t st);
int halo_masses(Ctx& c, const BoxParams& b, const HaloDev& h, const HostTables& tab, float* Mh_dev,
                int* count_dev, int* xc_dev, cudaStream_t st);
int flags_to_reference(const HaloDev& h, size_t ng, int64_t* out_dev, cudaStream_t st);

}  // namespace exh
