// The reference's file formats: parameter file, meta.txt, the six binary
// measurement files of a dataset directory, and the float64 grid / fft / image
// dumps and timing line.  Declared in include/wstack_gb300_io.h, which lists
// the formats and the reference lines each function replaces.
//
// Reading and writing are host work bounded by the file system; the device
// part is wsg_plan_dump_cube, which splits a resident cube into real and
// imaginary float64 planes on the GPU and overlaps the download of one chunk
// with the file write of the previous one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <string>
#include <vector>

#include "plan.cuh"
#include "wstack_gb300_io.h"

using namespace wsg;

namespace {

// ---------------------------------------------------------------------------
// small file helpers
// ---------------------------------------------------------------------------

struct File {
    FILE *f = nullptr;
    File(const char *path, const char *mode) : f(fopen(path, mode)) {}
    ~File()
    {
        if (f) fclose(f);
    }
    File(const File &) = delete;
    File &operator=(const File &) = delete;
    // fclose reports errors of buffered writes; call it explicitly after writing.
    bool close()
    {
        if (!f) return true;
        int r = fclose(f);
        f = nullptr;
        return r == 0;
    }
};

bool slurp(const char *path, std::string &out)
{
    File fp(path, "rb");
    if (!fp.f) return false;
    out.clear();
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), fp.f)) > 0) out.append(buf, n);
    return !ferror(fp.f);
}

bool copy_field(char *dst, size_t cap, const std::string &v)
{
    if (v.size() >= cap) return false;
    memcpy(dst, v.c_str(), v.size() + 1);
    return true;
}

// atoi(): leading whitespace, optional sign, decimal digits; 0 without digits.
int c_atoi(const std::string &s)
{
    errno = 0;
    long v = strtol(s.c_str(), nullptr, 10);
    if (v > INT_MAX) return INT_MAX;
    if (v < INT_MIN) return INT_MIN;
    return (int)v;
}

std::string joined(const char *dir, const char *name)
{
    std::string s(dir ? dir : "");
    s += name ? name : "";
    return s;
}

// ---------------------------------------------------------------------------
// device cube -> planar float64 chunks
// ---------------------------------------------------------------------------

template <typename C>
__global__ void k_split_cube(const C *__restrict__ cube, double *__restrict__ re,
                             double *__restrict__ im, long long n, double scale)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const C v = cube[i];
        re[i] = (double)v.x * scale;
        im[i] = (double)v.y * scale;
    }
}

}  // namespace

extern "C" {

int wsg_read_parameter_file(const char *path, wsg_params *out)
{
    clear_error();
    if (!path || !out) return set_error(WSG_ERR_ARG, "NULL argument");
    memset(out, 0, sizeof(*out));
    std::string text;
    if (!slurp(path, text)) return set_error(WSG_ERR_IO, "error opening paramfile %s", path);

    // whitespace-separated tokens (fscanf "%s")
    std::vector<std::string> tok;
    for (size_t i = 0; i < text.size();) {
        while (i < text.size() && isspace((unsigned char)text[i])) ++i;
        size_t j = i;
        while (j < text.size() && !isspace((unsigned char)text[j])) ++j;
        if (j > i) tok.emplace_back(text, i, j - i);
        i = j;
    }

    struct NameKey {
        const char *key;
        char *dst;
    };
    const NameKey names[] = {
        {"ufile", out->ufile},         {"vfile", out->vfile},
        {"wfile", out->wfile},         {"weightsfile", out->weightsfile},
        {"visrealfile", out->visrealfile}, {"visimgfile", out->visimgfile},
        {"metafile", out->metafile},   {"outfile", out->outfile},
        {"outfile1", out->outfile1},   {"outfile2", out->outfile2},
        {"outfile3", out->outfile3},   {"fftfile", out->fftfile},
        {"fftfile2", out->fftfile2},   {"fftfile3", out->fftfile3},
        {"logfile", out->logfile},     {"extension", out->extension},
        {"timingfile", out->timingfile},
    };

    // fscanf("%s%s", key, value) in a loop: a lone trailing key keeps the
    // previous value, and the loop ends when not even a key is left.
    std::string key, value;
    int filled = 1;   // the reference's counter i (init.c:130)
    for (size_t t = 0; t < tok.size(); t += 2) {
        key = tok[t];
        if (t + 1 < tok.size()) value = tok[t + 1];
        if (key == "num_threads") out->num_threads = c_atoi(value);
        if (key == "Datapath1") {
            if (!copy_field(out->datapath[0], WSG_PATH_LEN, value))
                return set_error(WSG_ERR_ARG, "paramfile %s: Datapath1 longer than %d characters",
                                 path, WSG_PATH_LEN - 1);
            ++filled;
        }
        if (key == "ndatasets") out->ndatasets = c_atoi(value);
        if (key == "w_support") out->w_support = c_atoi(value);
        if (key == "grid_size_x") out->grid_size_x = c_atoi(value);
        if (key == "grid_size_y") out->grid_size_y = c_atoi(value);
        if (key == "num_w_planes") out->num_w_planes = c_atoi(value);
        for (const NameKey &nk : names)
            if (key == nk.key && !copy_field(nk.dst, WSG_NAME_LEN, value))
                return set_error(WSG_ERR_ARG, "paramfile %s: %s longer than %d characters", path,
                                 nk.key, WSG_NAME_LEN - 1);
        if (key == "verbose_level") out->verbose_level = c_atoi(key);  // sic, init.c:233-236
        if (out->ndatasets > 1 && key == "Datapath" + std::to_string(filled)) {
            if (filled > WSG_MAX_DATASETS)
                return set_error(WSG_ERR_ARG, "paramfile %s: more than %d dataset directories",
                                 path, WSG_MAX_DATASETS);
            if (!copy_field(out->datapath[filled - 1], WSG_PATH_LEN, value))
                return set_error(WSG_ERR_ARG, "paramfile %s: %s longer than %d characters", path,
                                 key.c_str(), WSG_PATH_LEN - 1);
            ++filled;
        }
    }
    out->n_datapaths = filled - 1 < WSG_MAX_DATASETS ? filled - 1 : WSG_MAX_DATASETS;
    return WSG_OK;
}

int wsg_read_metadata(const char *path, wsg_metadata *out)
{
    clear_error();
    if (!path || !out) return set_error(WSG_ERR_ARG, "NULL argument");
    memset(out, 0, sizeof(*out));
    std::string text;
    if (!slurp(path, text)) return set_error(WSG_ERR_IO, "error opening meta file %s", path);

    static const char *const kNames[12] = {"Nmeasures", "Nvis",    "freq_per_chan", "polarisations",
                                          "Ntimes",    "dt",      "thours",        "baselines",
                                          "uvmin",     "uvmax",   "wmin",          "wmax"};
    long *const ints[12] = {&out->Nmeasures, &out->Nvis, &out->freq_per_chan, &out->polarisations,
                            &out->Ntimes, nullptr, nullptr, &out->baselines,
                            nullptr, nullptr, nullptr, nullptr};
    double *const dbls[12] = {nullptr, nullptr, nullptr, nullptr, nullptr, &out->dt, &out->thours,
                              nullptr, &out->uvmin, &out->uvmax, &out->wmin, &out->wmax};
    const char *p = text.c_str();
    for (int k = 0; k < 12; ++k) {
        char *end = nullptr;
        errno = 0;
        if (ints[k]) {
            long v = strtol(p, &end, 10);
            if (end == p)
                return set_error(WSG_ERR_IO, "meta file %s: field %d (%s) is not an integer", path,
                                 k + 1, kNames[k]);
            *ints[k] = v;
        } else {
            double v = strtod(p, &end);
            if (end == p)
                return set_error(WSG_ERR_IO, "meta file %s: field %d (%s) is not a number", path,
                                 k + 1, kNames[k]);
            *dbls[k] = v;
        }
        p = end;
    }
    return WSG_OK;
}

int wsg_partition_measurements(wsg_metadata *m, int rank, int size, long *startrow)
{
    clear_error();
    if (!m || !startrow) return set_error(WSG_ERR_ARG, "NULL argument");
    if (size < 1 || rank < 0 || rank >= size)
        return set_error(WSG_ERR_ARG, "rank %d outside [0, %d)", rank, size);
    if (m->freq_per_chan <= 0 || m->polarisations <= 0)
        return set_error(WSG_ERR_ARG, "freq_per_chan and polarisations must be positive");
    if (m->Nmeasures < WSG_DROPPED_ROWS)
        return set_error(WSG_ERR_ARG, "meta file lists %ld measurements, fewer than the %d dropped",
                         m->Nmeasures, WSG_DROPPED_ROWS);
    const long total = m->Nmeasures - WSG_DROPPED_ROWS;
    long per = total / size;
    const long rem = total % size;
    *startrow = (long)rank * per;
    if (rank == size - 1) per += rem;
    m->Nmeasures = per;
    m->Nvis = per * m->freq_per_chan * m->polarisations;
    m->Nweights = per * m->polarisations;
    return WSG_OK;
}

int wsg_read_measurements(const wsg_params *prm, int dataset, const wsg_metadata *m, long startrow,
                          double *uu, double *vv, double *ww, float *weights, float *vis_real,
                          float *vis_img)
{
    clear_error();
    if (!prm || !m) return set_error(WSG_ERR_ARG, "NULL argument");
    if (dataset < 0 || dataset >= WSG_MAX_DATASETS)
        return set_error(WSG_ERR_ARG, "dataset %d outside [0, %d)", dataset, WSG_MAX_DATASETS);
    if (m->Nmeasures < 0 || startrow < 0 || m->polarisations <= 0 || m->freq_per_chan <= 0)
        return set_error(WSG_ERR_ARG, "invalid measurement counts");
    if (m->Nmeasures > 0 && (!uu || !vv || !ww || !weights || !vis_real || !vis_img))
        return set_error(WSG_ERR_ARG, "NULL buffer");
    const char *dir = prm->datapath[dataset];

    struct Job {
        const char *what;      // the reference's word in its "error opening" messages
        std::string path;
        void *dst;
        size_t elem;
        long long count;
        long long offset;      // bytes
    };
    const long long pol = m->polarisations, fp = m->freq_per_chan * m->polarisations;
    Job jobs[6] = {
        {"ucoord", joined(dir, prm->ufile), uu, 8, m->Nmeasures, startrow * 8ll},
        {"vcoord", joined(dir, prm->vfile), vv, 8, m->Nmeasures, startrow * 8ll},
        {"wcoord", joined(dir, prm->wfile), ww, 8, m->Nmeasures, startrow * 8ll},
        {"weights", joined(dir, prm->weightsfile), weights, 4, m->Nweights, startrow * pol * 4},
        {"visibilities real", joined(dir, prm->visrealfile), vis_real, 4, m->Nvis, startrow * fp * 4},
        {"visibilities img", joined(dir, prm->visimgfile), vis_img, 4, m->Nvis, startrow * fp * 4},
    };
    // 0 = read in full, 1 = cannot open, 2 = short
    auto read_one = [](const Job &j) -> int {
        File fp(j.path.c_str(), "rb");
        if (!fp.f) return 1;
        if (j.count <= 0) return 0;
        size_t got = 0;
        if (fseeko(fp.f, (off_t)j.offset, SEEK_SET) == 0)
            got = fread(j.dst, j.elem, (size_t)j.count, fp.f);
        if ((long long)got == j.count) return 0;
        memset(static_cast<char *>(j.dst) + got * j.elem, 0, ((size_t)j.count - got) * j.elem);
        return 2;
    };
    std::future<int> fut[6];
    for (int k = 0; k < 6; ++k) fut[k] = std::async(std::launch::async, read_one, std::cref(jobs[k]));
    int res[6];
    for (int k = 0; k < 6; ++k) res[k] = fut[k].get();
    for (int k = 0; k < 6; ++k)
        if (res[k] == 1)
            return set_error(WSG_ERR_IO, "error opening %s file %s", jobs[k].what,
                             jobs[k].path.c_str());
    for (int k = 0; k < 6; ++k)
        if (res[k] == 2)
            return set_error(WSG_ERR_IO, "an error occurred while reading file %s",
                             jobs[k].path.c_str());
    return WSG_OK;
}

int wsg_reference_resolution(double uvmin, double uvmax, double *resolution)
{
    clear_error();
    if (!resolution) return set_error(WSG_ERR_ARG, "NULL argument");
    // abs(int): the double argument is converted to int (toward zero) first
    for (double v : {uvmin, uvmax})
        if (!(v > (double)INT_MIN - 1.0 && v < (double)INT_MAX + 1.0))
            return set_error(WSG_ERR_ARG, "uv limit %g outside the int range of abs()", v);
    const int a = abs((int)uvmin), b = abs((int)uvmax);
    *resolution = 1.0 / (double)(a > b ? a : b);
    return WSG_OK;
}

int wsg_write_cube_dump(const double *cube, int planes, int ny, int nx, double scale,
                        const char *real_path, const char *img_path)
{
    clear_error();
    if (!cube || !real_path || !img_path) return set_error(WSG_ERR_ARG, "NULL argument");
    if (planes <= 0 || ny <= 0 || nx <= 0) return set_error(WSG_ERR_ARG, "sizes must be positive");
    File fr(real_path, "wb"), fi(img_path, "wb");
    if (!fr.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", real_path);
    if (!fi.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", img_path);
    const long long n = (long long)planes * ny * nx;
    const long long chunk = 1ll << 20;
    std::vector<double> re((size_t)(n < chunk ? n : chunk)), im(re.size());
    for (long long i0 = 0; i0 < n; i0 += chunk) {
        const long long c = n - i0 < chunk ? n - i0 : chunk;
        for (long long i = 0; i < c; ++i) {
            re[i] = cube[2 * (i0 + i)] * scale;
            im[i] = cube[2 * (i0 + i) + 1] * scale;
        }
        if (fwrite(re.data(), sizeof(double), (size_t)c, fr.f) != (size_t)c)
            return set_error(WSG_ERR_IO, "write to %s failed", real_path);
        if (fwrite(im.data(), sizeof(double), (size_t)c, fi.f) != (size_t)c)
            return set_error(WSG_ERR_IO, "write to %s failed", img_path);
    }
    if (!fr.close()) return set_error(WSG_ERR_IO, "closing %s failed", real_path);
    if (!fi.close()) return set_error(WSG_ERR_IO, "closing %s failed", img_path);
    return WSG_OK;
}

int wsg_plan_dump_cube(wsg_plan *p, const void *cube, double scale, const char *real_path,
                       const char *img_path)
{
    clear_error();
    if (!p || !cube || !real_path || !img_path) return set_error(WSG_ERR_ARG, "NULL argument");
    File fr(real_path, "wb"), fi(img_path, "wb");
    if (!fr.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", real_path);
    if (!fi.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", img_path);

    const long long n = p->cube_planes() * p->npix();
    const long long chunk = n < (8ll << 20) ? n : (8ll << 20);   // 128 MiB of float64 pairs
    DevBuf stage;
    WSG_CUDA(stage.ensure(2 * 2 * (size_t)chunk * sizeof(double)));
    double *host = nullptr;
    WSG_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&host), 2 * 2 * (size_t)chunk * sizeof(double),
                           cudaHostAllocDefault));
    cudaEvent_t done[2] = {nullptr, nullptr};
    // writer[b] appends the chunk held in slot b; each writer first waits for
    // the one before it, so chunks reach the files in order
    std::shared_future<int> writer[2];
    int status = WSG_OK;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((chunk + threads - 1) / threads, 152ll * 8);

    // the writer of slot b: wait for its download, append both halves
    auto write_slot = [&](int b, long long c) -> int {
        if (cudaEventSynchronize(done[b]) != cudaSuccess) return WSG_ERR_CUDA;
        const double *re = host + (size_t)b * 2 * chunk;
        const double *im = re + chunk;
        if (fwrite(re, sizeof(double), (size_t)c, fr.f) != (size_t)c) return WSG_ERR_IO;
        if (fwrite(im, sizeof(double), (size_t)c, fi.f) != (size_t)c) return WSG_ERR_IO;
        return WSG_OK;
    };

    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2 && e == cudaSuccess; ++b)
        e = cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming);
    for (long long i0 = 0, k = 0; e == cudaSuccess && status == WSG_OK && i0 < n; i0 += chunk, ++k) {
        const int b = (int)(k & 1);
        const long long c = n - i0 < chunk ? n - i0 : chunk;
        if (writer[b].valid()) status = writer[b].get();   // slot b's previous chunk is on disk
        if (status != WSG_OK) break;
        double *dre = stage.as<double>() + (size_t)b * 2 * chunk;
        double *dim = dre + chunk;
        if (p->prec == WSG_FP64)
            k_split_cube<double2><<<blocks, threads, 0, p->stream>>>(
                static_cast<const double2 *>(cube) + i0, dre, dim, c, scale);
        else
            k_split_cube<float2><<<blocks, threads, 0, p->stream>>>(
                static_cast<const float2 *>(cube) + i0, dre, dim, c, scale);
        e = cudaGetLastError();
        double *hre = host + (size_t)b * 2 * chunk;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hre, dre, (size_t)c * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hre + chunk, dim, (size_t)c * sizeof(double), cudaMemcpyDeviceToHost,
                                p->stream);
        if (e == cudaSuccess) e = cudaEventRecord(done[b], p->stream);
        if (e == cudaSuccess) {
            std::shared_future<int> prev = writer[b ^ 1];
            writer[b] = std::async(std::launch::async, [&write_slot, prev, b, c]() {
                            if (prev.valid()) {
                                const int s = prev.get();
                                if (s != WSG_OK) return s;
                            }
                            return write_slot(b, c);
                        }).share();
        }
    }
    for (int b = 0; b < 2; ++b)
        if (writer[b].valid()) {
            int s = writer[b].get();
            if (status == WSG_OK) status = s;
        }
    for (int b = 0; b < 2; ++b)
        if (done[b]) cudaEventDestroy(done[b]);
    cudaFreeHost(host);
    if (e != cudaSuccess)
        return set_error(WSG_ERR_CUDA, "wsg_plan_dump_cube: %s", cudaGetErrorString(e));
    if (status == WSG_ERR_CUDA) return set_error(WSG_ERR_CUDA, "wsg_plan_dump_cube: download failed");
    if (status != WSG_OK) return set_error(WSG_ERR_IO, "write to %s / %s failed", real_path, img_path);
    if (!fr.close()) return set_error(WSG_ERR_IO, "closing %s failed", real_path);
    if (!fi.close()) return set_error(WSG_ERR_IO, "closing %s failed", img_path);
    return WSG_OK;
}

int wsg_write_image_dump(const double *image_real, const double *image_imag, long npix,
                         const char *real_path, const char *img_path)
{
    clear_error();
    if (!image_real || !image_imag || !real_path || !img_path)
        return set_error(WSG_ERR_ARG, "NULL argument");
    if (npix <= 0) return set_error(WSG_ERR_ARG, "npix must be positive");
    File fr(real_path, "wb"), fi(img_path, "wb");
    if (!fr.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", real_path);
    if (!fi.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", img_path);
    if (fwrite(image_real, sizeof(double), (size_t)npix, fr.f) != (size_t)npix)
        return set_error(WSG_ERR_IO, "write to %s failed", real_path);
    if (fwrite(image_imag, sizeof(double), (size_t)npix, fi.f) != (size_t)npix)
        return set_error(WSG_ERR_IO, "write to %s failed", img_path);
    if (!fr.close()) return set_error(WSG_ERR_IO, "closing %s failed", real_path);
    if (!fi.close()) return set_error(WSG_ERR_IO, "closing %s failed", img_path);
    return WSG_OK;
}

int wsg_write_timings(const char *path, const double s[7])
{
    clear_error();
    if (!path || !s) return set_error(WSG_ERR_ARG, "NULL argument");
    File f(path, "w");
    if (!f.f) return set_error(WSG_ERR_IO, "cannot open %s for writing", path);
    if (fprintf(f.f, "%f %f %f %f %f %f %f\n", s[0], s[1], s[2], s[3], s[4], s[5], s[6]) < 0)
        return set_error(WSG_ERR_IO, "write to %s failed", path);
    if (!f.close()) return set_error(WSG_ERR_IO, "closing %s failed", path);
    return WSG_OK;
}

}  // extern "C"
