/*
 * lsmgpu on-disk formats: LSMLIB's binary Grid file and its data-array files,
 * read and written with LSMLIB's own function names and signatures, so files
 * move between LSMLIB runs (on any machine with the same byte order) and this
 * library unchanged.
 *
 * Formats (native byte order, no padding; LSMLIB_REAL is double):
 *  - Grid file (src/utils/lsm_grid.c:614-677, read :680-760): num_dims;
 *    x_lo[3], x_hi[3], x_lo_ghostbox[3], x_hi_ghostbox[3] (double);
 *    grid_dims[3], grid_dims_ghostbox[3] (int); dx[3] (double); num_gridpts;
 *    the ghost, fill, D1, D2 and D3 boxes (6 ints each, ilo ihi jlo jhi klo
 *    khi); num_nb_levels; mark_gb, mark_D1, mark_D2, mark_D3, mark_fb
 *    (unsigned char); beta, gamma (double) — 297 bytes.
 *  - Data array (src/utils/lsm_data_arrays.c:364-437): 3 ints (ghost-box
 *    dimensions) then the values, column-major.
 *  - 1-D data array (lsm_data_arrays.c:440-491): 1 int (count) then values.
 * A file name ending in .gz or .bz2 is decompressed in place before reading
 * and compressed again afterwards; zip_status GZIP or BZIP2 compresses a
 * written file (file_name + ".gz" / ".bz2"), as LSMLIB does.  The
 * (de)compressor runs as a child process (gzip / bzip2 found on PATH)
 * without a shell.
 *
 * Data arrays may live on the GPU: the write functions accept a device
 * pointer for `data` and stream it to the file through pinned buffers; the
 * lsmgpu_read_data_array_into call fills a caller's host or device buffer.
 * Failures record a status for lsmgpu_get_last_error (lsmgpu.h); LSMLIB's
 * functions print a message and go on, and these do the same for
 * compatibility of their return values.
 */
#ifndef LSMGPU_IO_H
#define LSMGPU_IO_H

#ifdef __cplusplus
extern "C" {
#endif

#define LSMGPU_NO_ZIP 0
#define LSMGPU_GZIP 1
#define LSMGPU_BZIP2 2

/* Same members, order and layout as LSMLIB's Grid (src/utils/lsm_grid.h:43-95,
 * double-precision build), so a Grid* from a program built against LSMLIB's
 * headers can be passed where an LsmgpuGrid* is expected. */
typedef struct LsmgpuGrid {
  int num_dims;
  double x_lo[3];
  double x_hi[3];
  double x_lo_ghostbox[3];
  double x_hi_ghostbox[3];
  int grid_dims[3];
  int grid_dims_ghostbox[3];
  double dx[3];
  int num_gridpts;
  int ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb;
  int ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb;
  int ilo_D1_fb, ihi_D1_fb, jlo_D1_fb, jhi_D1_fb, klo_D1_fb, khi_D1_fb;
  int ilo_D2_fb, ihi_D2_fb, jlo_D2_fb, jhi_D2_fb, klo_D2_fb, khi_D2_fb;
  int ilo_D3_fb, ihi_D3_fb, jlo_D3_fb, jhi_D3_fb, klo_D3_fb, khi_D3_fb;
  int num_nb_levels;
  unsigned char mark_gb, mark_D1, mark_D2, mark_D3, mark_fb;
  double beta, gamma;
} LsmgpuGrid;

/* Grid construction (src/utils/lsm_grid.c:36-321, 789-1036), so a program
 * written against LSMLIB's lsm_grid.h needs no LSMLIB object for its index
 * spaces.  `accuracy` is LSMLIB's LSMLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE:
 * 0 LOW (ENO1, 2 ghost cells), 1 MEDIUM (ENO2, 3), 2 HIGH (ENO3, 5),
 * 3 VERY_HIGH (WENO5, 4).  Structures come from calloc (release with
 * destroyGrid or free).  A dimension other than 2 or 3 is reported on
 * stderr and replaced by 2, as LSMLIB does. */
LsmgpuGrid *allocateGrid(void);                                                   /* lsm_grid.c:36  */
LsmgpuGrid *createGridSetDx(int num_dims, double dx, double *x_lo, double *x_hi, int accuracy); /* :51 */
LsmgpuGrid *createGridSetDxDyDz(int num_dims, double dx, double dy, double dz, double *x_lo, double *x_hi,
                                int accuracy);                                    /* lsm_grid.c:117 */
LsmgpuGrid *createGridSetGridDims(int num_dims, int *grid_dims, double *x_lo, double *x_hi,
                                  int accuracy);                                  /* lsm_grid.c:189 */
LsmgpuGrid *copyGrid(LsmgpuGrid *grid);                                           /* lsm_grid.c:253 */
void destroyGrid(LsmgpuGrid *grid);                                               /* lsm_grid.c:317 */
/* Index spaces (ghost box from 0, fill box, D1/D2/D3 fill boxes) for the
 * scheme's stencil reach; setIndexSpaceLimits also sets the narrow-band
 * level count, the marks and the widths beta, gamma (lsm_grid.c:987-1036). */
void setIndexSpaceLimitsCentral(LsmgpuGrid *grid);                                /* lsm_grid.c:789 */
void setIndexSpaceLimitsENO1(LsmgpuGrid *grid);                                   /* lsm_grid.c:832 */
void setIndexSpaceLimitsENO2(LsmgpuGrid *grid);                                   /* lsm_grid.c:874 */
void setIndexSpaceLimitsENO3(LsmgpuGrid *grid);                                   /* lsm_grid.c:918 */
void setIndexSpaceLimitsWENO5(LsmgpuGrid *grid);                                  /* lsm_grid.c:962 */
void setIndexSpaceLimits(int accuracy, LsmgpuGrid *grid);                         /* lsm_grid.c:987 */

/* Writes `grid` in the binary Grid format.  Replaces writeGridToBinaryFile
 * (src/utils/lsm_grid.c:614; C declaration src/utils/lsm_grid.h:313). */
void writeGridToBinaryFile(LsmgpuGrid *grid, char *file_name, int zip_status);

/* Reads a binary Grid file into a new zero-initialised structure (release it
 * with free()).  An unreadable or short file leaves the missing members zero
 * and records an error.  Replaces readGridFromBinaryFile (lsm_grid.c:680;
 * lsm_grid.h:336). */
LsmgpuGrid *readGridFromBinaryFile(char *file_name);

/* Writes grid->grid_dims_ghostbox and grid->num_gridpts values of `data`
 * (host or device memory).  Replaces writeDataArray (lsm_data_arrays.c:364;
 * lsm_data_arrays.h:190). */
void writeDataArray(double *data, LsmgpuGrid *grid, char *file_name, int zip_status);

/* Writes n[3] and n[0]*n[1]*n[2] values of `data` (host or device memory).
 * Replaces writeDataArrayNoGrid (lsm_data_arrays.c:381; lsm_data_arrays.h:218). */
void writeDataArrayNoGrid(double *data, int *n, char *file_name, int zip_status);

/* Reads a data-array file: stores its dimensions in grid_dims_ghostbox[3] and
 * returns a malloc'ed host array of their product (release with free()), or
 * NULL when the file cannot be read.  Replaces readDataArray
 * (lsm_data_arrays.c:402; lsm_data_arrays.h:244). */
double *readDataArray(int *grid_dims_ghostbox, char *file_name);

/* Writes num_elements and the values of `data` (host or device memory).
 * Replaces writeDataArray1d (lsm_data_arrays.c:440; lsm_data_arrays.h:268). */
void writeDataArray1d(double *data, int num_elements, char *file_name, int zip_status);

/* Reads a 1-D data-array file into a malloc'ed host array (NULL on failure).
 * Replaces readDataArray1d (lsm_data_arrays.c:458; lsm_data_arrays.h:291). */
double *readDataArray1d(int *num_elements, char *file_name);

/* Reads a data-array file into dst (host or device memory, at least
 * `capacity` doubles) and stores its dimensions in grid_dims_ghostbox[3].  A
 * device destination is filled through pinned buffers with the file reads
 * overlapping the copies; the call returns when the data is in place.
 * Returns an LSMGPU_* status (LSMGPU_ERR_CAPACITY, and nothing written, when
 * the array holds more than `capacity` values).  No counterpart in LSMLIB: it
 * lets a caller load a fixture straight into an existing GPU array. */
int lsmgpu_read_data_array_into(const char *file_name, int *grid_dims_ghostbox, double *dst,
                                long long capacity);

#ifdef __cplusplus
}
#endif

#endif /* LSMGPU_IO_H */
