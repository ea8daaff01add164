// ctx.h -- the context behind faces_ctx (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/faces_gb300.h"
#include "geom.cuh"
#include "kernels.cuh"
#include "rows_setup.cuh"

struct faces_ctx {
  // geometry, flags, device tables and launch plans of one field (all ranks)
  int L[3], m[3], n;
  unsigned flags;
  int nranks;
  long sjy, sjz, R, total;
  std::vector<int> nbr;       // [rank*27+dir]
  std::vector<long> msg_off;  // [rank*27+dir], -1: none
  std::vector<long> recv_off; // [rank*27+dir]: what the rank receives, -1: none
  long msg_total = 0;
  int *d_nbr = nullptr;
  long *d_off = nullptr;
  long *d_roff = nullptr;
  double *d_msg = nullptr;
  unsigned long long *d_scratch = nullptr;  // check: rank maxima, max, first, values
  unsigned long long *d_sync = nullptr;     // fused pack: [0] arrivals, [1] the wait's error bits
  int pack_wait_extra = 0;                  // test hook (faces_test_pack_wait)
  long pack_wait_polls = 1L << 22;          // the fused pack's wait bound (about a second)
  double *d_field = nullptr;                // faces_run_host's device copy
  // faces_run_host_many: two more device fields (jobs rotate over three),
  // the streams and the events that order uploads, shares and downloads
  double *d_field2 = nullptr, *d_field3 = nullptr;
  bool pipe_ready = false;
  cudaStream_t s_up = nullptr, s_down = nullptr, s_comp = nullptr;  // uploads, downloads, shares
  cudaEvent_t ev_up[3] = {}, ev_done[3] = {}, ev_free[3] = {};
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int chunk = 0, tpb = 0, order = -1;
  int sms = 0;       // multiprocessors of the device
  faces::RowPlan plan;   // row kernel
  faces::RowPlan tplan;  // tile kernel
  faces::SeamPlan splan{};  // seam kernel
  long tgrid = 0;    // tile kernel CTAs
  int variant = 0;   // the kernel (default, or set by faces_autotune): 0 the tile step
                     // (periodic or mixed), 1 the general tile step, 2 the row
                     // kernel, 3 the seam kernel

  faces::FieldDesc desc(double *u) const
  {
    faces::FieldDesc f;
    f.u = u;
    f.sjy = sjy; f.sjz = sjz; f.R = R;
    f.n = n;
    for (int a = 0; a < 3; a++) { f.m[a] = m[a]; f.L[a] = L[a]; }
    f.periodic = (flags & FACES_PERIODIC) ? 1 : 0;
    f.mode = (flags & FACES_MESSAGES) ? faces::kMessages : faces::kDirect;
    f.nranks = nranks;
    f.msg = d_msg;
    f.msg_off = d_off;
    f.recv_off = d_roff;
    f.nbr = d_nbr;
    return f;
  }
};


