/*
 * refio: runs the reference's own reader (init.c: read_parameter_file,
 * op_filename, readMetaData, metaData_calculation, allocate_memory, readData)
 * and v-slab sectoring (gridding.c: initialize_array) for one dataset and one
 * rank, and writes what they produced to an output directory.  With the
 * extra argument "grid" (one rank only) it then runs the reference's
 * gridding loop and grid dump writer (gridding.c: gridding_data,
 * write_gridded_data, compiled with WRITE_DATA) into the same directory.
 * Test infrastructure only: it pins the library's reader, sectoring and dump
 * writer, and the restatements in oracle/, against the reference itself.
 *
 *   refio PARAMFILE DATASET RANK SIZE OUTDIR [grid]
 *
 * OUTDIR receives:
 *   params.txt   one "key value" line per parameter and output name
 *   meta.txt     the 13 meta fields after metaData_calculation, then startrow
 *   uu.bin vv.bin ww.bin weights.bin visreal.bin visimg.bin   as read
 *   histo.txt    histo_send[0..nsectors] of initialize_array, nsectors = SIZE
 *   sectors.bin  sectorarray[0..nsectors] concatenated, int64
 *   with "grid": the grid dump files under the parameter file's outfile2 and
 *   outfile3 names (prefixed with the dataset index, as the reference does)
 * The reference's steps run in init()'s order (init.c:10-65); the parameter
 * and meta files are read as rank 0 (which reads them and broadcasts), the
 * partition and the binary files as rank RANK of SIZE.
 */
#include "allvars.h"
#include "proto.h"

static void dump(const char *dir, const char *name, const void *p, size_t elem, long n)
{
    char path[2048];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) { perror(path); exit(2); }
    if (n > 0) fwrite(p, elem, (size_t)n, f);
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc != 6 && !(argc == 7 && !strcmp(argv[6], "grid"))) {
        fprintf(stderr, "usage: refio PARAMFILE DATASET RANK SIZE OUTDIR [grid]\n");
        return 2;
    }
    const int grid_mode = argc == 7;
    const int index = atoi(argv[2]), rank = atoi(argv[3]);
    const char *outdir = argv[5];
    size = atoi(argv[4]);
    if (grid_mode && size != 1) {
        fprintf(stderr, "refio: grid mode runs one rank\n");
        return 2;
    }
    global_rank = 0;
    read_parameter_file(argv[1]);
    /* init.c:16-33 */
    dx = 1.0 / (double)param.grid_size_x;
    dw = 1.0 / (double)param.num_w_planes;
    w_supporth = (double)((param.w_support - 1) / 2) * dx;
    nsectors = size;
    xaxis = param.grid_size_x;
    yaxis = param.grid_size_y / nsectors;
    strcpy(datapath, param.datapath_multi[index]);
    sprintf(num_buf, "%d", index);
    op_filename();
    fileName(datapath, in.metafile);
    readMetaData(filename);
    global_rank = rank;
    metaData_calculation();
    allocate_memory();
    readData();

    char path[2048];
    snprintf(path, sizeof(path), "%s/params.txt", outdir);
    FILE *f = fopen(path, "w");
    if (!f) { perror(path); return 2; }
    fprintf(f, "num_threads %d\nndatasets %d\ngrid_size_x %d\ngrid_size_y %d\n"
               "num_w_planes %d\nw_support %d\nverbose_level %d\n",
            param.num_threads, param.ndatasets, param.grid_size_x, param.grid_size_y,
            param.num_w_planes, param.w_support, verbose_level);
    for (int i = 0; i < NFILES; ++i)
        if (param.datapath_multi[i][0]) fprintf(f, "datapath%d %s\n", i, param.datapath_multi[i]);
    fprintf(f, "ufile %s\nvfile %s\nwfile %s\nweightsfile %s\nvisrealfile %s\nvisimgfile %s\n"
               "metafile %s\n", in.ufile, in.vfile, in.wfile, in.weightsfile, in.visrealfile,
            in.visimgfile, in.metafile);
    fprintf(f, "outfile %s\noutfile1 %s\noutfile2 %s\noutfile3 %s\nfftfile %s\nfftfile2 %s\n"
               "fftfile3 %s\nlogfile %s\nextension %s\ntimingfile %s\n",
            out.outfile, out.outfile1, out.outfile2, out.outfile3, out.fftfile, out.fftfile2,
            out.fftfile3, out.logfile, out.extension, out.timingfile);
    fclose(f);

    snprintf(path, sizeof(path), "%s/meta.txt", outdir);
    f = fopen(path, "w");
    if (!f) { perror(path); return 2; }
    fprintf(f, "%ld %ld %ld %ld %ld %ld %.17g %.17g %ld %.17g %.17g %.17g %.17g %ld\n",
            metaData.Nmeasures, metaData.Nvis, metaData.Nweights, metaData.freq_per_chan,
            metaData.polarisations, metaData.Ntimes, metaData.dt, metaData.thours,
            metaData.baselines, metaData.uvmin, metaData.uvmax, metaData.wmin, metaData.wmax,
            startrow);
    fclose(f);
    dump(outdir, "uu.bin", data.uu, sizeof(double), metaData.Nmeasures);
    dump(outdir, "vv.bin", data.vv, sizeof(double), metaData.Nmeasures);
    dump(outdir, "ww.bin", data.ww, sizeof(double), metaData.Nmeasures);
    dump(outdir, "weights.bin", data.weights, sizeof(float), metaData.Nweights);
    dump(outdir, "visreal.bin", data.visreal, sizeof(float), metaData.Nvis);
    dump(outdir, "visimg.bin", data.visimg, sizeof(float), metaData.Nvis);

    initialize_array();
    snprintf(path, sizeof(path), "%s/histo.txt", outdir);
    f = fopen(path, "w");
    if (!f) { perror(path); return 2; }
    for (long s = 0; s <= nsectors; ++s) fprintf(f, "%ld\n", histo_send[s]);
    fclose(f);
    snprintf(path, sizeof(path), "%s/sectors.bin", outdir);
    f = fopen(path, "wb");
    if (!f) { perror(path); return 2; }
    for (long s = 0; s <= nsectors; ++s)
        if (histo_send[s] > 0) fwrite(sectorarray[s], sizeof(long), (size_t)histo_send[s], f);
    fclose(f);

    if (grid_mode) {
        /* gridding() = initialize_array() + gridding_data() (gridding.c:8-33);
           the lists were built above */
        gridding_data();
        if (chdir(outdir) != 0) { perror(outdir); return 2; }
        write_gridded_data();
    }
    return 0;
}
