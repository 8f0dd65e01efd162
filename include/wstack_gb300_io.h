/*
 * wstack_gb300_io.h -- the reference's input reader, result dumps and
 * driver, as a C ABI over the GB300 w-stacking library
 * (lofar_gb300/libwstack_gb300.so; the compute entry points are in
 * wstack_gb300.h).
 *
 * The reference reads one parameter file, then for each dataset a meta.txt
 * and six raw binary files from a directory (a ".binMS"), grids, transforms,
 * w-corrects and optionally dumps the grid, the transformed planes and the
 * image as raw float64 files (init.c, gridding.c, fourier_transform.c,
 * result.c, main.c).  These functions read and write exactly those formats:
 *
 *   meta.txt                 12 whitespace-separated numbers, in the order of
 *                            wsg_metadata below           (init.c:278-307)
 *   ufile, vfile, wfile      float64[Nmeasures], native byte order
 *   weightsfile              float32[Nmeasures][polarisations]
 *   visrealfile, visimgfile  float32[Nmeasures][freq_per_chan][polarisations]
 *                                                         (init.c:387-501)
 *   grid / fft dumps         two files, real parts and imaginary parts, each
 *                            float64[num_w_planes][grid_size_y][grid_size_x]
 *                                                (gridding.c:366-447,
 *                                                 fourier_transform.c:74-159)
 *   image dump               two files, float64[grid_size_y][grid_size_x]
 *                                                (fourier_transform.c:177-219)
 *   timing file              one line "%f %f %f %f %f %f %f\n": setup,
 *                            kernel, compose, reduce, fft, phase, total
 *                            seconds                      (result.c:49-62)
 *
 * Every function returns a wsg_status (wsg_status and wsg_precision are
 * declared in wstack_gb300.h) and records a message for
 * wstack_gb300_last_error_string().  None of them exits the process.
 */
#ifndef WSTACK_GB300_IO_H_
#define WSTACK_GB300_IO_H_

#include "wstack_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define WSG_MAX_DATASETS 100  /* NFILES, allvars.h:33                         */
#define WSG_PATH_LEN 1024     /* a dataset directory (the reference: 900)     */
#define WSG_NAME_LEN 256      /* a file name inside it (the reference: 30)    */
#define WSG_DROPPED_ROWS 1000 /* rows removed from the end, init.c:317-320    */

/*
 * The parameter file (init.c:124-250, struct parameter / ip / op in
 * allvars.h).  Unset numbers are 0 and unset names empty, as the reference's
 * zero-initialised globals.
 */
typedef struct {
    int num_threads;
    int ndatasets;
    int grid_size_x;
    int grid_size_y;
    int num_w_planes;
    int w_support;
    int verbose_level;                  /* always 0: the reference parses the
                                           key, not the value (init.c:233-236) */
    int n_datapaths;                    /* entries of datapath[] that were set */
    char datapath[WSG_MAX_DATASETS][WSG_PATH_LEN];
    /* input names, joined to a dataset directory by plain concatenation
       (fileName, init.c:266-269) */
    char ufile[WSG_NAME_LEN], vfile[WSG_NAME_LEN], wfile[WSG_NAME_LEN];
    char weightsfile[WSG_NAME_LEN], visrealfile[WSG_NAME_LEN], visimgfile[WSG_NAME_LEN];
    char metafile[WSG_NAME_LEN];
    /* output names; a run prefixes each with the dataset index
       (op_filename, init.c:67-121) */
    char outfile[WSG_NAME_LEN], outfile1[WSG_NAME_LEN], outfile2[WSG_NAME_LEN];
    char outfile3[WSG_NAME_LEN], fftfile[WSG_NAME_LEN], fftfile2[WSG_NAME_LEN];
    char fftfile3[WSG_NAME_LEN], logfile[WSG_NAME_LEN], extension[WSG_NAME_LEN];
    char timingfile[WSG_NAME_LEN];
} wsg_params;

/* meta.txt, with the fields in the reference's struct meta order
   (allvars.h:78-93).  Nweights is not in the file: it is set by
   wsg_partition_measurements. */
typedef struct {
    long Nmeasures;
    long Nvis;
    long Nweights;
    long freq_per_chan;
    long polarisations;
    long Ntimes;
    double dt;
    double thours;
    long baselines;
    double uvmin;
    double uvmax;
    double wmin;
    double wmax;
} wsg_metadata;

/*
 * Replaces read_parameter_file() (init.c:124-250).  The file is read as a
 * stream of (key, value) token pairs separated by any whitespace; unknown keys
 * are ignored; a key that appears twice keeps its last value.  Dataset
 * directories follow the reference's rule: "Datapath1" always fills entry 0,
 * and while ndatasets (as read so far) is above 1 the key "Datapath<i>" fills
 * entry i-1, where i counts the entries filled so far plus one.  A trailing
 * key without a value is paired with the previous value, as fscanf leaves it.
 * Errors: WSG_ERR_IO (cannot open), WSG_ERR_ARG (a value longer than its
 * field).  num_threads == 0 is accepted here; wsg_run_paramfile rejects it
 * (main.c:52-56).
 */
WSG_API int wsg_read_parameter_file(const char *path, wsg_params *out);

/*
 * Replaces readMetaData() (init.c:278-307): 12 numbers read in order as
 * long, long, long, long, long, double, double, long, double, double, double,
 * double (scanf %ld / %lf semantics: leading whitespace skipped, the longest
 * valid prefix taken).  Nweights is set to 0.  Errors: WSG_ERR_IO (cannot
 * open; a field missing or not a number -- the reference would carry on with
 * stale values).
 */
WSG_API int wsg_read_metadata(const char *path, wsg_metadata *out);

/*
 * Replaces metaData_calculation() (init.c:311-343) for rank `rank` of `size`:
 * drops the last WSG_DROPPED_ROWS rows, splits the rest into `size`
 * contiguous row ranges (the last rank takes the remainder) and rewrites
 * Nmeasures, Nvis = Nmeasures*freq_per_chan*polarisations and
 * Nweights = Nmeasures*polarisations for this rank.  *startrow receives the
 * rank's first row.  Errors: WSG_ERR_ARG (fewer than WSG_DROPPED_ROWS rows,
 * rank outside [0, size), non-positive channel or polarisation counts).
 */
WSG_API int wsg_partition_measurements(wsg_metadata *meta, int rank, int size, long *startrow);

/*
 * Replaces readData() (init.c:387-501): reads this rank's rows of the six
 * binary files of dataset `dataset` (path = params->datapath[dataset] + file
 * name) into caller buffers of meta->Nmeasures, meta->Nweights and meta->Nvis
 * elements, starting at row `startrow`.  The six files are read concurrently.
 * Buffers may be pinned (cudaHostAlloc) host memory so that a following
 * upload runs at full link speed.  Errors: WSG_ERR_IO when a file cannot be
 * opened (the reference exits); when a file is shorter than asked, the rest
 * of that buffer is zero-filled (the reference's calloc'd buffers), all six
 * files are still read, and WSG_ERR_IO is returned with the reference's
 * message ("an error occurred while reading file ...").
 */
WSG_API int wsg_read_measurements(const wsg_params *params, int dataset, const wsg_metadata *meta,
                                  long startrow, double *uu, double *vv, double *ww,
                                  float *weights, float *vis_real, float *vis_img);

/*
 * resolution = 1 / MAX(abs(uvmin), abs(uvmax)) with the C library's int
 * abs(), so both values are truncated toward zero first (gridding.c:160;
 * the reference is compiled as C).  Both truncating to 0 gives +inf, as in
 * the reference.  Errors: WSG_ERR_ARG when a value is outside the int range.
 */
WSG_API int wsg_reference_resolution(double uvmin, double uvmax, double *resolution);

/*
 * Writes a [planes][ny][nx] complex128 cube held in HOST memory (re, im
 * interleaved) as the reference's two planar float64 dump files, each value
 * multiplied by `scale` (1 for the grid dump; the cube is written as is).
 * Replaces the single-rank body of write_gridded_data() (gridding.c:366-447)
 * and write_fftw_data() (fourier_transform.c:74-159).
 */
WSG_API int wsg_write_cube_dump(const double *cube, int planes, int ny, int nx, double scale,
                                const char *real_path, const char *img_path);

/*
 * The same dump from a cube resident on the plan's device, in the plan's
 * precision (complex128 for WSG_FP64, complex64 for WSG_FP32C; complex64
 * values are widened to float64).  Plane by plane, a kernel splits the cube
 * into real and imaginary planes (times `scale`) in a device staging buffer,
 * the planes are copied into pinned host buffers, and a writer thread appends
 * them to the two files while the next plane is split and copied.  Returns
 * when both files are written and closed.
 */
WSG_API int wsg_plan_dump_cube(wsg_plan *plan, const void *cube, double scale,
                               const char *real_path, const char *img_path);

/*
 * Writes an image as the reference's two float64[ny][nx] dump files
 * (fourier_transform.c:177-219; the files are truncated first).
 */
WSG_API int wsg_write_image_dump(const double *image_real, const double *image_imag, long npix,
                                 const char *real_path, const char *img_path);

/* Writes the reference's timing line (result.c:49-62): seconds[7] = setup,
   kernel, compose, reduce, fft, phase, total. */
WSG_API int wsg_write_timings(const char *path, const double seconds[7]);

/* ------------------------------------------------------------------ */
/* Driver: the reference's main() over the GB300 path                  */
/* ------------------------------------------------------------------ */

typedef struct {
    int precision;          /* WSG_FP64 (the reference's arithmetic) or WSG_FP32C     */
    int write_data;         /* the reference's -DWRITE_DATA: grid and fft dumps        */
    int write_image;        /* the reference's -DWRITE_IMAGE: image dump (it reuses,
                               and so replaces, the fft dump's file names)            */
    int write_timings;      /* the timing file of result.c:49-62                      */
    int verbose;            /* print the reference's progress lines on stdout         */
    char outdir[WSG_PATH_LEN]; /* directory for the output files ("" = current)       */
} wsg_run_options;

typedef struct {
    int datasets;           /* datasets run                                           */
    long Nmeasures;         /* rows gridded (last dataset, after the dropped rows)     */
    long Nvis;              /* visibilities (last dataset)                             */
    double resolution;      /* the value passed to the w-correction (last dataset)     */
    long long dropped;      /* rows not gridded (all datasets): off the single v-slab
                               (|vv| >= 1, gridding.c:42-56) or w-plane outside the grid */
    /* wall-clock seconds, summed over datasets (the reference's wt_timing):
       setup = meta + reading the binary files; compose = upload + (plane, tile)
       binning; kernel = gridding; reduce = 0 (one resident grid); fft; phase =
       w-correction + image download; write = dump files; total */
    double setup, compose, kernel, reduce, fft, phase, write, total;
} wsg_run_report;

WSG_API void wsg_run_options_default(wsg_run_options *opt);

/*
 * Replaces main() (main.c:8-94) for one process on one GPU: reads the
 * parameter file and, for each of its ndatasets datasets, the meta file and
 * the binary files (drop-last-1000 rule, one rank), grids all rows on the
 * current CUDA device with the plan API (dx = 1/grid_size_x,
 * dw = 1/num_w_planes, init.c:16-17), transforms each plane (FFTW_BACKWARD
 * convention, scaled by 1/(grid_size_x*grid_size_y)), applies the
 * w-correction with resolution from wsg_reference_resolution and the meta
 * file's wmin/wmax, and writes the requested dump files into opt->outdir
 * under the names "<dataset index><name>" (op_filename, init.c:67-121).
 * Errors: any status of the functions above; WSG_ERR_ARG when num_threads is
 * 0 (main.c:52-56) or ndatasets is outside [1, WSG_MAX_DATASETS] or names a
 * dataset without a directory.  A short binary file is reported on stderr and
 * the run carries on with zeros, as the reference does.
 */
WSG_API int wsg_run_paramfile(const char *paramfile, const wsg_run_options *opt,
                              wsg_run_report *report);

#ifdef __cplusplus
}
#endif

#endif /* WSTACK_GB300_IO_H_ */
