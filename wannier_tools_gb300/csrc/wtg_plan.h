// Host-side launch arithmetic of the per-model spectrum path.  Plain C++ (no
// CUDA types), so that its limits can be checked on a machine without a GPU.
#pragma once

#include <climits>
#include <cstddef>

namespace wtg {

// Largest k chunk of one Fourier-sum launch: k_fourier's grid.z is
// ceil(kc / 8) and must stay within 65535.
constexpr long long FOURIER_MAX_KC = 65535LL * 8;

// k points per chunk of wtg_surface_spectrum.  A chunk's H00/H01 (32 Ndim^2
// bytes per k) must fit h_bytes_max; the Fourier kernel's grid bounds it; and
// the chunk's kc * nomega instances, plus the one extra ticket each of the
// grid_max persistent CTAs takes from the work counter when it finds no work
// left, must stay a valid int (the counter and instance indices are 32-bit).
// Returns 0 when no chunk fits (nomega alone beyond INT_MAX - grid_max, or a
// size < 1).
inline int spectrum_kchunk(long long nk, long long nomega, long long ndim, long long grid_max,
                           size_t h_bytes_max) {
  if (nk < 1 || nomega < 1 || ndim < 1 || grid_max < 1) return 0;
  const long long room = (long long)INT_MAX - grid_max;
  if (nomega > room) return 0;
  const long long hk = 32LL * ndim * ndim;
  long long kc = (long long)(h_bytes_max / (size_t)hk);
  if (kc < 1) kc = 1;
  if (kc > nk) kc = nk;
  if (kc > FOURIER_MAX_KC) kc = FOURIER_MAX_KC;
  if (kc > room / nomega) kc = room / nomega;
  return (int)kc;
}

}  // namespace wtg
