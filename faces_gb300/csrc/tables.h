// tables.h -- host construction of the neighbour and message tables of a
// virtual rank grid (used by faces_api.cu and the CPU replay of the kernels).
#pragma once

#include <vector>

#include "geom.cuh"

namespace faces {

// neighbor(dx,dy,dz) of gpu/v-26-messages/Faces.cc:92-103 for every rank and
// direction; -1 (MPI_PROC_NULL) outside a non-periodic grid; [r*27+13] = r
inline std::vector<int> neighbour_table(const int L[3], bool periodic)
{
  const int nr = L[0] * L[1] * L[2];
  std::vector<int> t(nr * 27, -1);
  for (int r = 0; r < nr; r++) {
    const int k[3] = {r % L[0], (r / L[0]) % L[1], r / (L[0] * L[1])};
    for (int dir = 0; dir < 27; dir++) {
      const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
      int q[3];
      bool ok = true;
      for (int a = 0; a < 3; a++) {
        q[a] = k[a] + d[a];
        if (q[a] < 0 || q[a] >= L[a]) {
          if (!periodic) ok = false;
          q[a] = (q[a] + L[a]) % L[a];
        }
      }
      t[r * 27 + dir] = ok ? (q[2] * L[1] + q[1]) * L[0] + q[0] : -1;
    }
  }
  return t;
}

// offsets of the send buffers: one per rank and direction with a neighbour
// (gpu/v-26-messages/Faces.cc:16-27), each rounded to 32 doubles (256 bytes);
// returns the total doubles
inline long message_offsets(const FieldDesc &f, const std::vector<int> &nbr, std::vector<long> &off)
{
  off.assign(nbr.size(), -1);
  long tot = 0;
  for (int r = 0; r < f.nranks; r++)
    for (int dir = 0; dir < 27; dir++) {
      if (dir == 13 || nbr[r * 27 + dir] < 0) continue;
      const int d[3] = {dir % 3 - 1, (dir / 3) % 3 - 1, dir / 9 - 1};
      off[r * 27 + dir] = tot;
      tot += (region_size(f, d) + 31) / 32 * 32;
    }
  return tot;
}

// offsets of what each rank receives: recv[r*27+dir] = the offset of
// neighbour(r,dir)'s buffer toward the opposite direction, -1 without one
inline std::vector<long> receive_offsets(const std::vector<int> &nbr, const std::vector<long> &off)
{
  std::vector<long> recv(nbr.size(), -1);
  for (size_t i = 0; i < nbr.size(); i++) {
    const int dir = (int)(i % 27), q = nbr[i];
    if (dir != 13 && q >= 0) recv[i] = off[q * 27 + (26 - dir)];
  }
  return recv;
}

}  // namespace faces
