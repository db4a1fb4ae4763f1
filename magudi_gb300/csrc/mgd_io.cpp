// mgd_io.cpp -- file formats around the hot path: PLOT3D whole-format
// multi-block grid and solution files (the layout of write_skeleton and the
// plot3dWriteSingle* routines, src/PLOT3DFormat.c:208-292,
// src/PLOT3DHelperImpl.f90:554-784: 4-byte record markers, native byte order,
// 5 solution components with the energy in the fifth slot, a 4-double
// auxiliary header per block) and the raw actuator-patch control/gradient
// streams (src/ActuatorPatchImpl.f90:226-458). Host code only: these
// functions need no GPU.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/magudi_gb300.h"

namespace {

struct File {
  FILE* f = nullptr;
  explicit File(const char* name, const char* mode) : f(std::fopen(name, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

bool putMarker(FILE* f, long long bytes) {
  const int32_t m = (int32_t)bytes;
  return (long long)m == bytes && std::fwrite(&m, 4, 1, f) == 1;
}

bool getMarker(FILE* f, long long* bytes) {
  int32_t m = 0;
  if (std::fread(&m, 4, 1, f) != 1) return false;
  *bytes = m;
  return true;
}

// Header: nGrids, then the grid sizes (3 per grid).
bool writeHeader(FILE* f, int nGrids, const int* sizes) {
  if (!putMarker(f, 4) || std::fwrite(&nGrids, 4, 1, f) != 1 || !putMarker(f, 4)) return false;
  const long long bytes = 12LL * nGrids;
  if (!putMarker(f, bytes)) return false;
  for (int i = 0; i < 3 * nGrids; ++i) {
    const int32_t s = sizes[i];
    if (std::fwrite(&s, 4, 1, f) != 1) return false;
  }
  return putMarker(f, bytes);
}

bool readHeader(FILE* f, int nGrids, const int* sizes) {
  long long m = 0, m2 = 0;
  int32_t n = 0;
  if (!getMarker(f, &m) || m != 4 || std::fread(&n, 4, 1, f) != 1 || !getMarker(f, &m2) || m2 != 4) return false;
  if (n != nGrids) return false;
  if (!getMarker(f, &m) || m != 12LL * nGrids) return false;
  for (int i = 0; i < 3 * nGrids; ++i) {
    int32_t s = 0;
    if (std::fread(&s, 4, 1, f) != 1 || s != sizes[i]) return false;
  }
  return getMarker(f, &m2) && m2 == m;
}

long long points(const int* s) { return (long long)s[0] * s[1] * s[2]; }

}  // namespace

int mgd_plot3d_write_grid(const char* filename, int n_grids, const int* grid_sizes, int n_dimensions,
                          const double* const* coordinates, const int* const* iblank) {
  File file(filename, "wb");
  if (!file.f || n_grids < 1 || n_dimensions < 1 || n_dimensions > 3) return 1;
  if (!writeHeader(file.f, n_grids, grid_sizes)) return 1;
  for (int g = 0; g < n_grids; ++g) {
    const long long N = points(grid_sizes + 3 * g);
    const long long bytes = (3 * 8 + 4) * N;
    if (!putMarker(file.f, bytes)) return 1;
    std::vector<double> zero((size_t)N, 0.0);
    for (int d = 0; d < 3; ++d) {
      const double* src = d < n_dimensions ? coordinates[g] + N * d : zero.data();
      if (std::fwrite(src, 8, (size_t)N, file.f) != (size_t)N) return 1;
    }
    std::vector<int32_t> ib((size_t)N, 1);
    if (iblank && iblank[g])
      for (long long p = 0; p < N; ++p) ib[(size_t)p] = iblank[g][p];
    if (std::fwrite(ib.data(), 4, (size_t)N, file.f) != (size_t)N || !putMarker(file.f, bytes)) return 1;
  }
  return 0;
}

int mgd_plot3d_write_solution(const char* filename, int n_grids, const int* grid_sizes, int n_components,
                              const double* const* q, const double* aux) {
  File file(filename, "wb");
  if (!file.f || n_grids < 1 || n_components < 3 || n_components > 5) return 1;
  if (!writeHeader(file.f, n_grids, grid_sizes)) return 1;
  for (int g = 0; g < n_grids; ++g) {
    const long long N = points(grid_sizes + 3 * g);
    if (!putMarker(file.f, 32) || std::fwrite(aux, 8, 4, file.f) != 4 || !putMarker(file.f, 32)) return 1;
    const long long bytes = 5 * 8 * N;
    if (!putMarker(file.f, bytes)) return 1;
    // components 1 .. n-1 in slots 1 .. n-1, the last one (energy) in slot 5
    std::vector<double> zero((size_t)N, 0.0);
    for (int slot = 0; slot < 5; ++slot) {
      const double* src = zero.data();
      if (slot < n_components - 1) src = q[g] + N * slot;
      else if (slot == 4) src = q[g] + N * (n_components - 1);
      if (std::fwrite(src, 8, (size_t)N, file.f) != (size_t)N) return 1;
    }
    if (!putMarker(file.f, bytes)) return 1;
  }
  return 0;
}

int mgd_plot3d_read_solution(const char* filename, int n_grids, const int* grid_sizes, int n_components,
                             double* const* q, double* aux) {
  File file(filename, "rb");
  if (!file.f || n_grids < 1 || n_components < 3 || n_components > 5) return 1;
  if (!readHeader(file.f, n_grids, grid_sizes)) return 1;
  for (int g = 0; g < n_grids; ++g) {
    const long long N = points(grid_sizes + 3 * g);
    long long m = 0;
    double a[4];
    if (!getMarker(file.f, &m) || m != 32 || std::fread(a, 8, 4, file.f) != 4 || !getMarker(file.f, &m)) return 1;
    if (aux && g == 0) std::memcpy(aux, a, sizeof a);
    if (!getMarker(file.f, &m) || m != 5 * 8 * N) return 1;
    std::vector<double> buf((size_t)N);
    for (int slot = 0; slot < 5; ++slot) {
      if (std::fread(buf.data(), 8, (size_t)N, file.f) != (size_t)N) return 1;
      double* dst = nullptr;
      if (slot < n_components - 1) dst = q[g] + N * slot;
      else if (slot == 4) dst = q[g] + N * (n_components - 1);
      if (dst) std::memcpy(dst, buf.data(), (size_t)N * 8);
    }
    if (!getMarker(file.f, &m)) return 1;
  }
  return 0;
}

int mgd_write_patch_stream(const char* filename, const double* entries, long long n_entries,
                           long long points_per_entry, long long stride, long long offset) {
  File file(filename, "wb");
  if (!file.f || n_entries < 0 || points_per_entry < 0) return 1;
  for (long long e = 0; e < n_entries; ++e)
    if (std::fwrite(entries + e * stride + offset, 8, (size_t)points_per_entry, file.f) != (size_t)points_per_entry)
      return 1;
  return 0;
}

int mgd_read_patch_stream(const char* filename, double* entries, long long n_entries, long long points_per_entry,
                          long long stride, long long offset) {
  File file(filename, "rb");
  if (!file.f || n_entries < 0 || points_per_entry < 0) return 1;
  for (long long e = 0; e < n_entries; ++e)
    if (std::fread(entries + e * stride + offset, 8, (size_t)points_per_entry, file.f) != (size_t)points_per_entry)
      return 1;
  return 0;
}
