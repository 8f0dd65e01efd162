/*
 * refio: runs the reference's own reader (init.c: read_parameter_file,
 * op_filename, readMetaData, metaData_calculation, allocate_memory, readData)
 * for one dataset and one rank, and writes what it read to an output
 * directory.  Test infrastructure only: it pins the library's reader
 * (wsg_read_parameter_file & co.) and the NumPy restatement in
 * oracle/binms_oracle.py against the reference itself.
 *
 *   refio PARAMFILE DATASET RANK SIZE OUTDIR
 *
 * OUTDIR receives:
 *   params.txt   one "key value" line per parameter and output name
 *   meta.txt     the 13 meta fields after metaData_calculation, then startrow
 *   uu.bin vv.bin ww.bin weights.bin visreal.bin visimg.bin   as read
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
    if (argc != 6) {
        fprintf(stderr, "usage: refio PARAMFILE DATASET RANK SIZE OUTDIR\n");
        return 2;
    }
    const int index = atoi(argv[2]), rank = atoi(argv[3]);
    const char *outdir = argv[5];
    size = atoi(argv[4]);
    global_rank = 0;
    read_parameter_file(argv[1]);
    xaxis = param.grid_size_x;
    yaxis = param.grid_size_y / size;
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
    return 0;
}
