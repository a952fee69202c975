// LSMLIB's binary Grid and data-array files (src/utils/lsm_grid.c:614-760,
// src/utils/lsm_data_arrays.c:364-491, compression src/utils/lsm_file.c),
// read and written with LSMLIB's function names, plus a loader that fills a
// device array directly.
//
// Host arrays go through one fwrite / fread.  Device arrays are streamed
// through two pinned buffers: while one chunk is written to (or read from)
// the file, the next is copied between the device and the other buffer on
// the library stream, so the disk and the PCIe / C2C link work at the same
// time.  The pinned buffers are allocated on first use and kept.
#include <spawn.h>
#include <sys/wait.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "lsmgpu_common.cuh"
#include "../../include/lsmgpu_io.h"

extern char **environ;

namespace lsmgpu {
namespace {

constexpr size_t kGridRecordBytes = 297;
constexpr size_t kChunkBytes = size_t(32) << 20;  // per pinned buffer

// Runs `tool flag path` as a child process (no shell) and waits for it.
bool run_tool(const char *tool, const char *flag, const std::string &path) {
  pid_t pid;
  char *argv[] = {const_cast<char *>(tool), const_cast<char *>(flag), const_cast<char *>(path.c_str()), nullptr};
  if (posix_spawnp(&pid, tool, nullptr, nullptr, argv, environ) != 0) return false;
  int status = 0;
  if (waitpid(pid, &status, 0) < 0) return false;
  return WIFEXITED(status) && WEXITSTATUS(status) == 0;
}

bool ends_with(const std::string &s, const char *suffix) {
  const size_t n = strlen(suffix);
  return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// Decompresses name in place when it ends in .gz / .bz2 (lsm_file.c:19-53);
// returns the uncompressed name and the compression to restore afterwards.
bool unzip(const char *what, const char *name, std::string &base, int &zip) {
  base = name;
  zip = LSMGPU_NO_ZIP;
  if (ends_with(base, ".gz")) {
    zip = LSMGPU_GZIP;
    if (!run_tool("gzip", "-df", base)) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: gzip -d failed on %s", what, name);
      return false;
    }
    base.resize(base.size() - 3);
  } else if (ends_with(base, ".bz2")) {
    zip = LSMGPU_BZIP2;
    if (!run_tool("bzip2", "-df", base)) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: bzip2 -d failed on %s", what, name);
      return false;
    }
    base.resize(base.size() - 4);
  }
  return true;
}

// Compresses `base` (lsm_file.c:56-70); a failure is recorded.
void rezip(const char *what, const std::string &base, int zip) {
  if (zip == LSMGPU_GZIP && !run_tool("gzip", "-f", base))
    set_error(LSMGPU_ERR_ARGUMENT, "%s: gzip failed on %s", what, base.c_str());
  if (zip == LSMGPU_BZIP2 && !run_tool("bzip2", "-f", base))
    set_error(LSMGPU_ERR_ARGUMENT, "%s: bzip2 failed on %s", what, base.c_str());
}

FILE *open_or_fail(const char *what, const std::string &path, const char *mode) {
  FILE *fp = fopen(path.c_str(), mode);
  if (!fp) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: could not open file %s", what, path.c_str());
    fprintf(stderr, "lsmgpu: %s: could not open file %s\n", what, path.c_str());
  }
  return fp;
}

bool on_device(const void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();  // no device, or a plain host pointer
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

struct Pinned {
  std::mutex mu;
  char *buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool ready = false;
  bool init(const char *what) {
    if (ready) return true;
    for (int b = 0; b < 2; b++) {
      if (cudaMallocHost((void **)&buf[b], kChunkBytes) != cudaSuccess ||
          cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        set_error(LSMGPU_ERR_CUDA, "%s: cannot allocate the pinned staging buffers", what);
        return false;
      }
    }
    ready = true;
    return true;
  }
};
Pinned &pinned() {
  static Pinned p;
  return p;
}

// fwrite n doubles from host or device memory
bool write_values(const char *what, FILE *fp, const double *data, long long n) {
  if (n <= 0) return true;
  if (!data) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null data pointer", what);
    return false;
  }
  if (!on_device(data)) {
    if ((long long)fwrite(data, sizeof(double), (size_t)n, fp) != n) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
      return false;
    }
    return true;
  }
  Pinned &P = pinned();
  std::lock_guard<std::mutex> lock(P.mu);
  if (!P.init(what)) return false;
  const long long per = (long long)(kChunkBytes / sizeof(double));
  const long long nchunks = (n + per - 1) / per;
  auto issue = [&](long long c) {
    const long long off = c * per, cnt = (n - off < per) ? n - off : per;
    cudaMemcpyAsync(P.buf[c & 1], data + off, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost, stream());
    cudaEventRecord(P.ev[c & 1], stream());
  };
  issue(0);
  bool ok = true;
  for (long long c = 0; c < nchunks; c++) {
    if (c + 1 < nchunks) issue(c + 1);  // its buffer was written to the file in step c - 1
    if (!cuda_ok(cudaEventSynchronize(P.ev[c & 1]), what)) return false;
    const long long off = c * per, cnt = (n - off < per) ? n - off : per;
    if (ok && (long long)fwrite(P.buf[c & 1], sizeof(double), (size_t)cnt, fp) != cnt) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
      ok = false;
    }
  }
  return ok && cuda_ok(cudaGetLastError(), what);
}

// fread n doubles into host or device memory
bool read_values(const char *what, FILE *fp, double *dst, long long n) {
  if (n <= 0) return true;
  if (!on_device(dst)) {
    if ((long long)fread(dst, sizeof(double), (size_t)n, fp) != n) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: file shorter than its header says", what);
      return false;
    }
    return true;
  }
  Pinned &P = pinned();
  std::lock_guard<std::mutex> lock(P.mu);
  if (!P.init(what)) return false;
  const long long per = (long long)(kChunkBytes / sizeof(double));
  bool ok = true;
  for (long long c = 0, off = 0; off < n; c++, off += per) {
    const long long cnt = (n - off < per) ? n - off : per;
    if (c >= 2 && !cuda_ok(cudaEventSynchronize(P.ev[c & 1]), what)) return false;  // copy c - 2 is done
    if ((long long)fread(P.buf[c & 1], sizeof(double), (size_t)cnt, fp) != cnt) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: file shorter than its header says", what);
      ok = false;
      break;
    }
    cudaMemcpyAsync(dst + off, P.buf[c & 1], (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice, stream());
    cudaEventRecord(P.ev[c & 1], stream());
  }
  return cuda_ok(cudaStreamSynchronize(stream()), what) && ok;
}

// Grid record in file order (lsm_grid.c:619-673)
struct Rec {
  unsigned char b[kGridRecordBytes];
  size_t at = 0;
  template <class T> void put(const T *v, int n) {
    memcpy(b + at, v, sizeof(T) * n);
    at += sizeof(T) * n;
  }
  template <class T> void get(T *v, int n, size_t have) {
    for (int q = 0; q < n; q++, at += sizeof(T))
      if (at + sizeof(T) <= have) memcpy(v + q, b + at, sizeof(T));
  }
};

// packs the grid into r (have == 0) or unpacks the first `have` bytes of r
void walk(Rec &r, LsmgpuGrid *g, size_t have) {
  auto f = [&](auto *v, int n) {
    if (have == 0)
      r.put(v, n);
    else
      r.get(v, n, have);
  };
  f(&g->num_dims, 1);
  f(g->x_lo, 3); f(g->x_hi, 3); f(g->x_lo_ghostbox, 3); f(g->x_hi_ghostbox, 3);
  f(g->grid_dims, 3); f(g->grid_dims_ghostbox, 3);
  f(g->dx, 3);
  f(&g->num_gridpts, 1);
  f(&g->ilo_gb, 1); f(&g->ihi_gb, 1); f(&g->jlo_gb, 1); f(&g->jhi_gb, 1); f(&g->klo_gb, 1); f(&g->khi_gb, 1);
  f(&g->ilo_fb, 1); f(&g->ihi_fb, 1); f(&g->jlo_fb, 1); f(&g->jhi_fb, 1); f(&g->klo_fb, 1); f(&g->khi_fb, 1);
  f(&g->ilo_D1_fb, 1); f(&g->ihi_D1_fb, 1); f(&g->jlo_D1_fb, 1); f(&g->jhi_D1_fb, 1); f(&g->klo_D1_fb, 1);
  f(&g->khi_D1_fb, 1);
  f(&g->ilo_D2_fb, 1); f(&g->ihi_D2_fb, 1); f(&g->jlo_D2_fb, 1); f(&g->jhi_D2_fb, 1); f(&g->klo_D2_fb, 1);
  f(&g->khi_D2_fb, 1);
  f(&g->ilo_D3_fb, 1); f(&g->ihi_D3_fb, 1); f(&g->jlo_D3_fb, 1); f(&g->jhi_D3_fb, 1); f(&g->klo_D3_fb, 1);
  f(&g->khi_D3_fb, 1);
  f(&g->num_nb_levels, 1);
  f(&g->mark_gb, 1); f(&g->mark_D1, 1); f(&g->mark_D2, 1); f(&g->mark_D3, 1); f(&g->mark_fb, 1);
  f(&g->beta, 1); f(&g->gamma, 1);
}

// dimensions header of a data array: three ints, their product
bool read_dims(const char *what, FILE *fp, int *dims, int ndims, long long &n) {
  if ((int)fread(dims, sizeof(int), (size_t)ndims, fp) != ndims) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: file too short for its header", what);
    return false;
  }
  n = 1;
  for (int d = 0; d < ndims; d++) {
    if (dims[d] < 0) {
      set_error(LSMGPU_ERR_ARGUMENT, "%s: negative dimension in the header", what);
      return false;
    }
    n *= dims[d];
  }
  return true;
}

}  // namespace
}  // namespace lsmgpu

using namespace lsmgpu;

extern "C" {

void writeGridToBinaryFile(LsmgpuGrid *grid, char *file_name, int zip_status) {
  const char *what = "writeGridToBinaryFile";
  clear_error();
  if (!grid || !file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return;
  }
  Rec r;
  walk(r, grid, 0);
  FILE *fp = open_or_fail(what, file_name, "wb");
  if (!fp) return;
  const bool ok = fwrite(r.b, 1, kGridRecordBytes, fp) == kGridRecordBytes;
  fclose(fp);
  if (!ok) set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
  rezip(what, file_name, zip_status);
}

// ---- Grid construction -------------------------------------------------
// Ghost cells per accuracy level: LOW (ENO1) 2, MEDIUM (ENO2) 3, HIGH (ENO3)
// 5, VERY_HIGH (WENO5) 4 (lsm_grid.c:47).
static int grid_ghost_cells(int accuracy) {
  static const int g[4] = {2, 3, 5, 4};
  return (accuracy >= 0 && accuracy < 4) ? g[accuracy] : g[1];
}

LsmgpuGrid *allocateGrid(void) { return (LsmgpuGrid *)calloc(1, sizeof(LsmgpuGrid)); }

void destroyGrid(LsmgpuGrid *grid) { free(grid); }

LsmgpuGrid *copyGrid(LsmgpuGrid *grid) {
  LsmgpuGrid *g = allocateGrid();
  if (g && grid) *g = *grid;
  return g;
}

static int grid_dims_of(int num_dims, const char *what) {
  if (num_dims == 2 || num_dims == 3) return num_dims;
  fprintf(stderr, "\n%s: invalid number of dimensions (%d), set to 2.\n", what, num_dims);
  set_error(LSMGPU_ERR_ARGUMENT, "%s: invalid number of dimensions (%d), set to 2", what, num_dims);
  return 2;
}

// ghost-box extents from the interior ones; the third axis of a 2D grid is
// one cell with zero extent and spacing (lsm_grid.c:90-108)
static void grid_finish(LsmgpuGrid *g, int accuracy) {
  const int ng = grid_ghost_cells(accuracy);
  g->num_gridpts = 1;
  for (int i = 0; i < g->num_dims; i++) {
    g->grid_dims_ghostbox[i] = g->grid_dims[i] + 2 * ng;
    g->x_lo_ghostbox[i] = g->x_lo[i] - ng * g->dx[i];
    g->x_hi_ghostbox[i] = g->x_hi[i] + ng * g->dx[i];
    g->num_gridpts *= g->grid_dims_ghostbox[i];
  }
  if (g->num_dims == 2) {
    g->x_lo[2] = 0;
    g->x_hi[2] = 0;
    g->x_lo_ghostbox[2] = 0;
    g->x_hi_ghostbox[2] = 0;
    g->grid_dims[2] = 1;
    g->grid_dims_ghostbox[2] = 1;
    g->dx[2] = 0;
  }
  setIndexSpaceLimits(accuracy, g);
}

// spacing given: the cell count is the nearest integer to the extent over
// the spacing, and x_hi moves to x_lo + cells * spacing (lsm_grid.c:82-88)
static LsmgpuGrid *grid_from_spacing(int num_dims, const double sp[3], const double *x_lo, const double *x_hi,
                                     int accuracy, const char *what) {
  LsmgpuGrid *g = allocateGrid();
  if (!g) return nullptr;
  g->num_dims = grid_dims_of(num_dims, what);
  for (int i = 0; i < 3; i++) g->dx[i] = sp[i];
  for (int i = 0; i < g->num_dims; i++) {
    g->grid_dims[i] = (int)rint((x_hi[i] - x_lo[i]) / g->dx[i]);
    g->x_lo[i] = x_lo[i];
    g->x_hi[i] = x_lo[i] + g->grid_dims[i] * g->dx[i];
  }
  grid_finish(g, accuracy);
  return g;
}

LsmgpuGrid *createGridSetDx(int num_dims, double dx, double *x_lo, double *x_hi, int accuracy) {
  clear_error();
  const double sp[3] = {dx, dx, num_dims == 3 ? dx : 0.0};
  LsmgpuGrid *g = grid_from_spacing(num_dims, sp, x_lo, x_hi, accuracy, "createGridSetDx");
  if (g && g->num_dims == 3) g->dx[2] = dx;
  return g;
}

LsmgpuGrid *createGridSetDxDyDz(int num_dims, double dx, double dy, double dz, double *x_lo, double *x_hi,
                                int accuracy) {
  clear_error();
  const double sp[3] = {dx, dy, dz};
  return grid_from_spacing(num_dims, sp, x_lo, x_hi, accuracy, "createGridSetDxDyDz");
}

// cell counts given: the spacing is the extent over the count (lsm_grid.c:216)
LsmgpuGrid *createGridSetGridDims(int num_dims, int *grid_dims, double *x_lo, double *x_hi, int accuracy) {
  clear_error();
  LsmgpuGrid *g = allocateGrid();
  if (!g) return nullptr;
  g->num_dims = grid_dims_of(num_dims, "createGridSetGridDims");
  for (int i = 0; i < g->num_dims; i++) {
    g->grid_dims[i] = grid_dims[i];
    g->x_hi[i] = x_hi[i];
    g->x_lo[i] = x_lo[i];
    g->dx[i] = (g->x_hi[i] - g->x_lo[i]) / g->grid_dims[i];
  }
  grid_finish(g, accuracy);
  return g;
}

// ghost box from 0; the D1 / D2 / D3 fill boxes lose 1 / 2 / 3 cells per
// side (lsm_grid.c:789-812)
void setIndexSpaceLimitsCentral(LsmgpuGrid *g) {
  int *gb[3][2] = {{&g->ilo_gb, &g->ihi_gb}, {&g->jlo_gb, &g->jhi_gb}, {&g->klo_gb, &g->khi_gb}};
  int *d1[3][2] = {{&g->ilo_D1_fb, &g->ihi_D1_fb}, {&g->jlo_D1_fb, &g->jhi_D1_fb}, {&g->klo_D1_fb, &g->khi_D1_fb}};
  int *d2[3][2] = {{&g->ilo_D2_fb, &g->ihi_D2_fb}, {&g->jlo_D2_fb, &g->jhi_D2_fb}, {&g->klo_D2_fb, &g->khi_D2_fb}};
  int *d3[3][2] = {{&g->ilo_D3_fb, &g->ihi_D3_fb}, {&g->jlo_D3_fb, &g->jhi_D3_fb}, {&g->klo_D3_fb, &g->khi_D3_fb}};
  for (int a = 0; a < 3; a++) {
    const int top = g->grid_dims_ghostbox[a] - 1;
    *gb[a][0] = 0; *gb[a][1] = top;
    *d1[a][0] = 1; *d1[a][1] = top - 1;
    *d2[a][0] = 2; *d2[a][1] = top - 2;
    *d3[a][0] = 3; *d3[a][1] = top - 3;
  }
}

// fill box = the cells where both the plus and the minus derivative are
// defined: minus from D_lo + lo_shift, plus up to D_hi - hi_shift
static void fill_box_from(LsmgpuGrid *g, int order, int lo_shift, int hi_shift) {
  setIndexSpaceLimitsCentral(g);
  const int lo[3] = {order == 1 ? g->ilo_D1_fb : order == 2 ? g->ilo_D2_fb : g->ilo_D3_fb,
                     order == 1 ? g->jlo_D1_fb : order == 2 ? g->jlo_D2_fb : g->jlo_D3_fb,
                     order == 1 ? g->klo_D1_fb : order == 2 ? g->klo_D2_fb : g->klo_D3_fb};
  const int hi[3] = {order == 1 ? g->ihi_D1_fb : order == 2 ? g->ihi_D2_fb : g->ihi_D3_fb,
                     order == 1 ? g->jhi_D1_fb : order == 2 ? g->jhi_D2_fb : g->jhi_D3_fb,
                     order == 1 ? g->khi_D1_fb : order == 2 ? g->khi_D2_fb : g->khi_D3_fb};
  g->ilo_fb = lo[0] + lo_shift; g->ihi_fb = hi[0] - hi_shift;
  g->jlo_fb = lo[1] + lo_shift; g->jhi_fb = hi[1] - hi_shift;
  g->klo_fb = lo[2] + lo_shift; g->khi_fb = hi[2] - hi_shift;
}

void setIndexSpaceLimitsENO1(LsmgpuGrid *g) { fill_box_from(g, 1, 0, 1); }   // lsm_grid.c:832-865
void setIndexSpaceLimitsENO2(LsmgpuGrid *g) { fill_box_from(g, 2, 1, 1); }   // :874-909
void setIndexSpaceLimitsENO3(LsmgpuGrid *g) { fill_box_from(g, 3, 1, 2); }   // :918-953
void setIndexSpaceLimitsWENO5(LsmgpuGrid *g) { fill_box_from(g, 1, 2, 3); }  // :962-985

// marks 120 (ghost box), 119, 118, 117 (D1-D3), 120 - levels (fill box);
// beta / gamma 3 / 6 cells above MEDIUM accuracy, else 2 / 4 (:987-1036)
void setIndexSpaceLimits(int accuracy, LsmgpuGrid *g) {
  g->mark_gb = 120;
  g->mark_D1 = (unsigned char)(g->mark_gb - 1);
  g->mark_D2 = (unsigned char)(g->mark_gb - 2);
  g->mark_D3 = (unsigned char)(g->mark_gb - 3);
  g->num_nb_levels = grid_ghost_cells(accuracy);
  g->mark_fb = (unsigned char)(g->mark_gb - g->num_nb_levels);
  if (accuracy > 1) {
    g->beta = 3 * g->dx[0];
    g->gamma = 6 * g->dx[0];
  } else {
    g->beta = 2 * g->dx[0];
    g->gamma = 4 * g->dx[0];
  }
  switch (accuracy) {
    case 0: setIndexSpaceLimitsENO1(g); break;
    case 2: setIndexSpaceLimitsENO3(g); break;
    case 3: setIndexSpaceLimitsWENO5(g); break;
    default: setIndexSpaceLimitsENO2(g);
  }
}

LsmgpuGrid *readGridFromBinaryFile(char *file_name) {
  const char *what = "readGridFromBinaryFile";
  clear_error();
  LsmgpuGrid *grid = (LsmgpuGrid *)calloc(1, sizeof(LsmgpuGrid));
  if (!file_name || !grid) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return grid;
  }
  std::string base;
  int zip;
  if (!unzip(what, file_name, base, zip)) return grid;
  FILE *fp = open_or_fail(what, base, "rb");
  if (!fp) return grid;
  Rec r;
  const size_t have = fread(r.b, 1, kGridRecordBytes, fp);
  fclose(fp);
  if (have > 0) walk(r, grid, have);
  if (have < kGridRecordBytes) set_error(LSMGPU_ERR_ARGUMENT, "%s: %s holds %zu of 297 bytes", what, base.c_str(), have);
  rezip(what, base, zip);
  return grid;
}

void writeDataArray(double *data, LsmgpuGrid *grid, char *file_name, int zip_status) {
  const char *what = "writeDataArray";
  clear_error();
  if (!grid || !file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return;
  }
  FILE *fp = open_or_fail(what, file_name, "wb");
  if (!fp) return;
  bool ok = fwrite(grid->grid_dims_ghostbox, sizeof(int), 3, fp) == 3;
  ok = ok && write_values(what, fp, data, grid->num_gridpts);
  fclose(fp);
  if (!ok && lsmgpu_get_last_error(nullptr, 0) == LSMGPU_OK) set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
  rezip(what, file_name, zip_status);
}

void writeDataArrayNoGrid(double *data, int *n, char *file_name, int zip_status) {
  const char *what = "writeDataArrayNoGrid";
  clear_error();
  if (!n || !file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return;
  }
  FILE *fp = open_or_fail(what, file_name, "wb");
  if (!fp) return;
  bool ok = fwrite(n, sizeof(int), 3, fp) == 3;
  ok = ok && write_values(what, fp, data, (long long)n[0] * n[1] * n[2]);
  fclose(fp);
  if (!ok && lsmgpu_get_last_error(nullptr, 0) == LSMGPU_OK) set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
  rezip(what, file_name, zip_status);
}

double *readDataArray(int *grid_dims_ghostbox, char *file_name) {
  const char *what = "readDataArray";
  clear_error();
  if (!grid_dims_ghostbox || !file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return nullptr;
  }
  std::string base;
  int zip;
  if (!unzip(what, file_name, base, zip)) return nullptr;
  FILE *fp = open_or_fail(what, base, "rb");
  if (!fp) return nullptr;
  long long n = 0;
  double *data = nullptr;
  if (read_dims(what, fp, grid_dims_ghostbox, 3, n)) {
    data = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (!data) {
      set_error(LSMGPU_ERR_CAPACITY, "%s: cannot allocate %lld values", what, n);
    } else if (!read_values(what, fp, data, n)) {
      free(data);
      data = nullptr;
    }
  }
  fclose(fp);
  rezip(what, base, zip);
  return data;
}

void writeDataArray1d(double *data, int num_elements, char *file_name, int zip_status) {
  const char *what = "writeDataArray1d";
  clear_error();
  if (!file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return;
  }
  FILE *fp = open_or_fail(what, file_name, "wb");
  if (!fp) return;
  bool ok = fwrite(&num_elements, sizeof(int), 1, fp) == 1;
  ok = ok && write_values(what, fp, data, num_elements);
  fclose(fp);
  if (!ok && lsmgpu_get_last_error(nullptr, 0) == LSMGPU_OK) set_error(LSMGPU_ERR_ARGUMENT, "%s: short write", what);
  rezip(what, file_name, zip_status);
}

double *readDataArray1d(int *num_elements, char *file_name) {
  const char *what = "readDataArray1d";
  clear_error();
  if (!num_elements || !file_name) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return nullptr;
  }
  std::string base;
  int zip;
  if (!unzip(what, file_name, base, zip)) return nullptr;
  FILE *fp = open_or_fail(what, base, "rb");
  if (!fp) return nullptr;
  long long n = 0;
  double *data = nullptr;
  if (read_dims(what, fp, num_elements, 1, n)) {
    data = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (!data) {
      set_error(LSMGPU_ERR_CAPACITY, "%s: cannot allocate %lld values", what, n);
    } else if (!read_values(what, fp, data, n)) {
      free(data);
      data = nullptr;
    }
  }
  fclose(fp);
  rezip(what, base, zip);
  return data;
}

int lsmgpu_read_data_array_into(const char *file_name, int *grid_dims_ghostbox, double *dst, long long capacity) {
  const char *what = "lsmgpu_read_data_array_into";
  clear_error();
  if (!file_name || !grid_dims_ghostbox || !dst) {
    set_error(LSMGPU_ERR_ARGUMENT, "%s: null argument", what);
    return LSMGPU_ERR_ARGUMENT;
  }
  std::string base;
  int zip;
  if (!unzip(what, file_name, base, zip)) return LSMGPU_ERR_ARGUMENT;
  FILE *fp = open_or_fail(what, base, "rb");
  if (!fp) return LSMGPU_ERR_ARGUMENT;
  long long n = 0;
  if (read_dims(what, fp, grid_dims_ghostbox, 3, n)) {
    if (n > capacity)
      set_error(LSMGPU_ERR_CAPACITY, "%s: %s holds %lld values, the buffer %lld", what, base.c_str(), n, capacity);
    else
      read_values(what, fp, dst, n);
  }
  fclose(fp);
  const int status = lsmgpu_get_last_error(nullptr, 0);
  rezip(what, base, zip);
  return status != LSMGPU_OK ? status : lsmgpu_get_last_error(nullptr, 0);
}

}  // extern "C"
