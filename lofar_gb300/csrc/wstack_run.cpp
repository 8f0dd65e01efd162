// wstack_gb300_run: the reference's executable (main.c:8-94) on one GPU.
//
//   wstack_gb300_run PARAMFILE [--write-data] [--write-image] [--fp32c]
//                    [--outdir DIR] [--no-timings] [--quiet]
//
// The reference chooses its dumps at compile time (-DWRITE_DATA,
// -DWRITE_IMAGE, Makefile:35-37); here they are flags.  Exit status 1 on any
// error, with the library's message on stderr, as the reference exits 1 when
// a file cannot be opened.
#include <cstdio>
#include <cstring>

#include "wstack_gb300_io.h"

int main(int argc, char **argv)
{
    wsg_run_options opt;
    wsg_run_options_default(&opt);
    opt.verbose = 1;
    const char *paramfile = nullptr;
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (!strcmp(a, "--write-data")) {
            opt.write_data = 1;
        } else if (!strcmp(a, "--write-image")) {
            opt.write_image = 1;
        } else if (!strcmp(a, "--fp32c")) {
            opt.precision = WSG_FP32C;
        } else if (!strcmp(a, "--no-timings")) {
            opt.write_timings = 0;
        } else if (!strcmp(a, "--quiet")) {
            opt.verbose = 0;
        } else if (!strcmp(a, "--outdir") && i + 1 < argc) {
            if (strlen(argv[i + 1]) >= sizeof(opt.outdir)) {
                fprintf(stderr, "--outdir longer than %zu characters\n", sizeof(opt.outdir) - 1);
                return 1;
            }
            strcpy(opt.outdir, argv[++i]);
        } else if (a[0] == '-' || paramfile) {
            fprintf(stderr, "unknown argument %s\n", a);
            return 1;
        } else {
            paramfile = a;
        }
    }
    if (!paramfile) {
        fprintf(stderr, "Parameter file is not given\n");
        return 1;
    }
    wsg_run_report rep;
    const int st = wsg_run_paramfile(paramfile, &opt, &rep);
    if (st != WSG_OK) {
        fprintf(stderr, "wstack_gb300_run: %s\n", wstack_gb300_last_error_string());
        return 1;
    }
    if (opt.verbose) printf("*************************************************************\n");
    return 0;
}
