// faces_main.cc -- the `faces` executable: drop-in for the reference's
// benchmark driver gpu/main.cc:108-199 on one GB300.
//
// stdin : lx ly lz mx my mz n nk nj ni   (gpu/main.cc:137-138); ni < 0 runs
//         shares without the compute (inner) kernels (gpu/main.cc:157-161)
// stdout: the reference's lines (gpu/main.cc:139-143,104,194 and the Faces
//         constructor line gpu/v-26-messages/Faces.cc:79-81).  The lx*ly*lz
//         MPI ranks are virtual ranks in one GPU, so the MPI reductions of the
//         time become one value: avg = min = max.
// The correctness check compares every rank's field with the closed form of
// ni shares of the initial state on the GPU (faces_check) instead of running
// the host Mugs oracle; "N tasks passed correctness check" counts the ranks
// whose maximum relative error is below 1e-15 (gpu/main.cc:39-105).
//
// Options (argv, so the stdin contract is unchanged):
//   --periodic        wrap the rank grid (the reference never wraps)
//   --messages        v-26 strategy: 26 messages per rank, swapped by buffer
//   --gather          force the generic one-thread-per-point kernel
//   --rows            use the register row kernel instead of the tile kernel
//   --v6              v-6 strategy: six face messages per rank, sweeps z, y, x
//   --v6f             the same in the fused form (four launches per share)
//   --general         periodic fields: the general tile step
//   --init=ref|int    initial state: gpu/main.cc:18 formula (default) or
//                     integer values from --seed=S
//   --chunk=K --tpb=T --order=O   work decomposition (faces_set_tuning)
//   --autotune        pick the kernel and its settings on the field before the
//                     timed loop (faces_autotune; the field is re-initialised
//                     before each timed loop, as always)
//   --json            one machine-readable line on stderr
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/faces_gb300.h"

namespace {

void die(const char *what, int rc)
{
  std::fprintf(stderr, "FACES ERROR %d in %s: %s\n", rc, what, faces_last_error());
  std::fflush(stderr);
  std::exit(1);
}

#define TRY(call)                          \
  do {                                     \
    const int rc_ = (call);                \
    if (rc_ != FACES_OK) die(#call, rc_);  \
  } while (0)

void cuda_check(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return;
  std::fprintf(stderr, "GPU ERROR in %s: %s %s\n", what, cudaGetErrorName(e), cudaGetErrorString(e));
  std::fflush(stderr);
  std::exit(1);
}

}  // namespace

int main(int argc, char *argv[])
{
  unsigned flags = 0;
  int init = 0, chunk = 0, tpb = 0, order = -1;
  bool json = false, autotune = false;
  unsigned long long seed = 1;
  for (int a = 1; a < argc; a++) {
    const std::string s = argv[a];
    if (s == "--periodic") flags |= FACES_PERIODIC;
    else if (s == "--messages") flags |= FACES_MESSAGES;
    else if (s == "--gather") flags |= FACES_GATHER;
    else if (s == "--rows") flags |= FACES_ROWS;
    else if (s == "--seams") flags |= FACES_SEAMS;
    else if (s == "--v6") flags |= FACES_V6;
    else if (s == "--v6f") flags |= FACES_V6F;
    else if (s == "--general") flags |= FACES_GENERAL;
    else if (s == "--json") json = true;
    else if (s == "--autotune") autotune = true;
    else if (s == "--init=ref") init = 0;
    else if (s == "--init=int") init = 1;
    else if (s.rfind("--seed=", 0) == 0) seed = std::strtoull(s.c_str() + 7, nullptr, 10);
    else if (s.rfind("--chunk=", 0) == 0) chunk = std::atoi(s.c_str() + 8);
    else if (s.rfind("--tpb=", 0) == 0) tpb = std::atoi(s.c_str() + 6);
    else if (s.rfind("--order=", 0) == 0) order = std::atoi(s.c_str() + 8);
    else {
      std::fprintf(stderr, "unknown option %s\n", argv[a]);
      return 2;
    }
  }

  int lx, ly, lz, mx, my, mz, n, niface, niel, nshare;
  if (!(std::cin >> lx >> ly >> lz >> mx >> my >> mz >> n >> niface >> niel >> nshare)) {
    std::fprintf(stderr, "expected 10 integers on stdin: lx ly lz mx my mz n nk nj ni\n");
    return 2;
  }
  std::cout << lx << ' ' << ly << ' ' << lz << " tasks\n";
  std::cout << mx << ' ' << my << ' ' << mz << " local elements of size " << n << '\n';
  std::cout << niface << " face inits x " << niel << " element inits x ";
  if (nshare < 0) std::cout << -nshare << " shares without compute kernels" << std::endl;
  else std::cout << nshare << " shares" << std::endl;

  bool compute = true;
  if (nshare < 0) {
    compute = false;
    nshare = -nshare;
  }

  // the field outlives the Faces objects (gpu/main.cc:169)
  faces_ctx *layout = nullptr;
  TRY(faces_create(&layout, lx, ly, lz, mx, my, mz, n, flags));
  double *u = nullptr;
  TRY(faces_field_alloc(layout, &u));
  const int nranks = lx * ly * lz;

  double t = 0;
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  float gpu_ms = 0;
  for (int k = 0; k < niface; k++) {
    std::cout << (k + 1) << ": ";
    faces_ctx *faces = nullptr;
    TRY(faces_create(&faces, lx, ly, lz, mx, my, mz, n, flags));
    if (chunk > 0 || tpb > 0 || order >= 0) TRY(faces_set_tuning(faces, chunk, tpb, order));
    if (autotune) {
      TRY(faces_init_int(faces, u, seed, nullptr));
      const int applied = faces_autotune(faces, u, compute ? 1 : 0, 3, nullptr);
      if (applied < 0) TRY(applied);
    }
    std::cout << "Initialized Faces: " << mx << " x " << my << " x " << mz << " elements of order " << n - 1
              << " on " << lx << " x " << ly << " x " << lz << " tasks" << std::endl;
    for (int j = 0; j <= niel; j++) {
      if (init == 0) TRY(faces_init_ref(faces, u, nullptr));
      else TRY(faces_init_int(faces, u, seed, nullptr));
      cuda_check(cudaDeviceSynchronize(), "init");
      const auto tstart = std::chrono::steady_clock::now();
      cuda_check(cudaEventRecord(e0, nullptr), "cudaEventRecord");
      TRY(faces_share_n(faces, u, compute ? 1 : 0, nshare, nullptr));
      cuda_check(cudaEventRecord(e1, nullptr), "cudaEventRecord");
      cuda_check(cudaDeviceSynchronize(), "share");
      const auto tstop = std::chrono::steady_clock::now();
      if (j > 0) {
        t += std::chrono::duration<double>(tstop - tstart).count();
        float ms = 0;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        gpu_ms += ms;
      }
    }
    TRY(faces_destroy(faces));
  }

  std::vector<double> rank_max(nranks);
  double maxrel = 0, vals[2] = {0, 0};
  int npass = 0, where[7] = {0, 0, 0, 0, 0, 0, 0};
  TRY(faces_check(layout, u, init, seed, niface > 0 ? nshare : 0, compute ? 1 : 0, rank_max.data(), &maxrel, &npass,
                  where, vals, nullptr));
  for (int r = 0; r < nranks; r++) {
    if (rank_max[r] < 1e-15) continue;
    std::cout << r << " FAIL " << rank_max[r];
    if (r == where[0]) {
      const double ue = vals[0], ve = vals[1];
      std::cout << " (" << where[1];
      for (int i = 2; i < 7; i++) std::cout << ',' << where[i];
      std::cout << ") " << ue << ' ' << ve << ' ' << std::abs(ue - ve) << ' '
                << std::abs(ue - ve) / (std::abs(ue) + std::abs(ve));
    }
    std::cout << std::endl;
  }
  std::cout << npass << " tasks passed correctness check" << std::endl;
  std::cout << "time " << t << " avg " << t << " min " << t << " max" << std::endl;

  if (json) {
    long total = 0;
    TRY(faces_layout(layout, nullptr, nullptr, &total));
    const long points = (long)n * n * n * mx * my * mz * nranks;
    const long timed = (long)niface * niel * nshare;
    const double bytes = 16.0 * points * timed;
    std::fprintf(stderr,
                 "{\"points\": %ld, \"timed_shares\": %ld, \"wall_s\": %.9g, \"gpu_s\": %.9g, \"gbs_wall\": %.6g, "
                 "\"gbs_gpu\": %.6g, \"maxrel\": %.3g, \"npass\": %d, \"nranks\": %d}\n",
                 points, timed, t, gpu_ms * 1e-3, t > 0 ? bytes / t * 1e-9 : 0.0,
                 gpu_ms > 0 ? bytes / (gpu_ms * 1e-3) * 1e-9 : 0.0, maxrel, npass, nranks);
  }
  TRY(faces_field_free(u));
  TRY(faces_destroy(layout));
  return 0;
}
