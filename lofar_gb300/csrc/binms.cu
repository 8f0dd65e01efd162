// The reference's file formats: parameter file, meta.txt, the six binary
// measurement files of a dataset directory, and the float64 grid / fft / image
// dumps and timing line.  Declared in include/wstack_gb300_io.h, which lists
// the formats and the reference lines each function replaces.
//
// Reading and writing are host work bounded by the file system: the reader
// cuts the six files into chunks read by a pool of threads, and each dump
// writes its real and imaginary files from two threads.  The device part is
// wsg_plan_dump_cube, which splits a resident cube into real and imaginary
// float64 chunks on the GPU and overlaps the download of one chunk with the
// file writes of the previous one.
#include <cuda_runtime.h>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <string>
#include <thread>
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
// parallel reader: every file is cut into chunks that a pool of threads reads
// with pread, so the page cache (or the disk) is read with all cores; the
// part of a buffer beyond the end of a short file is zero-filled
// ---------------------------------------------------------------------------

constexpr long long kReadChunk = 32ll << 20;

struct ReadJob {
    const char *what;            // the reference's word in its "error opening" messages
    std::string path;
    void *dst;
    long long bytes;             // wanted
    long long offset;            // in the file
    int fd = -1;
    std::atomic<bool> short_read{false};
    ReadJob(const char *w, std::string p, void *d, long long b, long long o)
        : what(w), path(std::move(p)), dst(d), bytes(b), offset(o) {}
};

void read_parallel(ReadJob *jobs, int njobs)
{
    struct Piece {
        ReadJob *job;
        long long from, len;     // bytes of the destination
    };
    std::vector<Piece> pieces;
    for (int k = 0; k < njobs; ++k) {
        ReadJob &j = jobs[k];
        struct stat st;
        long long avail = 0;
        if (fstat(j.fd, &st) == 0) avail = std::max(0ll, (long long)st.st_size - j.offset);
        if (avail < j.bytes) {
            j.short_read = true;
            memset(static_cast<char *>(j.dst) + avail, 0, (size_t)(j.bytes - avail));
        }
        const long long have = std::min(avail, j.bytes);
        for (long long a = 0; a < have; a += kReadChunk)
            pieces.push_back({&j, a, std::min(kReadChunk, have - a)});
    }
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < pieces.size();) {
            const Piece &pc = pieces[i];
            char *dst = static_cast<char *>(pc.job->dst) + pc.from;
            long long done = 0;
            while (done < pc.len) {
                const ssize_t r = pread(pc.job->fd, dst + done, (size_t)(pc.len - done),
                                        (off_t)(pc.job->offset + pc.from + done));
                if (r <= 0) {   // the file shrank or failed under us: zero the rest
                    pc.job->short_read = true;
                    memset(dst + done, 0, (size_t)(pc.len - done));
                    break;
                }
                done += r;
            }
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nthreads = std::min<size_t>(std::min(16u, hw), pieces.size());
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (std::thread &t : pool) t.join();
}

// ---------------------------------------------------------------------------
// device cube -> planar float64 chunks
// ---------------------------------------------------------------------------

constexpr long long kDumpChunk = 8ll << 20;   // values per chunk of a device dump

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

cudaError_t wsg::launch_split_complex(const void *src, int prec, double *re, double *im,
                                      long long n, double scale, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 152ll * 8);
    if (prec == WSG_FP64)
        k_split_cube<double2><<<blocks, threads, 0, stream>>>(static_cast<const double2 *>(src), re,
                                                              im, n, scale);
    else
        k_split_cube<float2><<<blocks, threads, 0, stream>>>(static_cast<const float2 *>(src), re,
                                                             im, n, scale);
    return cudaGetLastError();
}

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
    const long long pol = m->polarisations, fp = m->freq_per_chan * m->polarisations;
    ReadJob jobs[6] = {
        {"ucoord", joined(dir, prm->ufile), uu, 8ll * m->Nmeasures, startrow * 8ll},
        {"vcoord", joined(dir, prm->vfile), vv, 8ll * m->Nmeasures, startrow * 8ll},
        {"wcoord", joined(dir, prm->wfile), ww, 8ll * m->Nmeasures, startrow * 8ll},
        {"weights", joined(dir, prm->weightsfile), weights, 4ll * m->Nweights, startrow * pol * 4},
        {"visibilities real", joined(dir, prm->visrealfile), vis_real, 4ll * m->Nvis,
         startrow * fp * 4},
        {"visibilities img", joined(dir, prm->visimgfile), vis_img, 4ll * m->Nvis,
         startrow * fp * 4},
    };
    // open in the reference's order: the first file that cannot be opened is reported
    for (ReadJob &j : jobs) {
        j.fd = open(j.path.c_str(), O_RDONLY);
        if (j.fd < 0) {
            for (ReadJob &k : jobs)
                if (k.fd >= 0) close(k.fd);
            return set_error(WSG_ERR_IO, "error opening %s file %s", j.what, j.path.c_str());
        }
    }
    read_parallel(jobs, 6);
    for (ReadJob &j : jobs) close(j.fd);
    for (const ReadJob &j : jobs)
        if (j.short_read.load())
            return set_error(WSG_ERR_IO, "an error occurred while reading file %s", j.path.c_str());
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
    // one thread per file: each takes its component of the interleaved cube
    auto write_part = [&](int part, FILE *f) -> bool {
        const long long chunk = 1ll << 20;
        std::vector<double> buf((size_t)std::min(n, chunk));
        for (long long i0 = 0; i0 < n; i0 += chunk) {
            const long long c = std::min(n - i0, chunk);
            for (long long i = 0; i < c; ++i) buf[i] = cube[2 * (i0 + i) + part] * scale;
            if (fwrite(buf.data(), sizeof(double), (size_t)c, f) != (size_t)c) return false;
        }
        return true;
    };
    auto im_ok = std::async(std::launch::async, write_part, 1, fi.f);
    const bool re_ok = write_part(0, fr.f);
    if (!im_ok.get()) return set_error(WSG_ERR_IO, "write to %s failed", img_path);
    if (!re_ok) return set_error(WSG_ERR_IO, "write to %s failed", real_path);
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
    const long long chunk = std::min(n, kDumpChunk);
    DevBuf stage;
    WSG_CUDA(stage.ensure(2 * 2 * (size_t)chunk * sizeof(double)));
    // two slots of (re, im) host staging; each file has its own chain of
    // writers, and each writer waits for the one before it on the same file,
    // so chunks reach the files in order while the next chunk is split and
    // downloaded
    std::vector<double> host[2];
    std::shared_future<bool> wre[2], wim[2];
    auto chain = [](std::shared_future<bool> prev, FILE *f, const double *src, long long c) {
        return std::async(std::launch::async, [prev, f, src, c]() {
                   if (prev.valid() && !prev.get()) return false;
                   return fwrite(src, sizeof(double), (size_t)c, f) == (size_t)c;
               }).share();
    };
    bool ok = true;
    cudaError_t e = cudaSuccess;
    for (long long i0 = 0, k = 0; ok && e == cudaSuccess && i0 < n; i0 += chunk, ++k) {
        const int b = (int)(k & 1);
        const long long c = std::min(n - i0, chunk);
        if (wre[b].valid()) ok = wre[b].get() && ok;   // slot b's last chunk is written
        if (wim[b].valid()) ok = wim[b].get() && ok;
        if (!ok) break;
        double *dre = stage.as<double>() + (size_t)b * 2 * chunk;
        double *dim = dre + chunk;
        e = launch_split_complex(static_cast<const char *>(cube) + (size_t)i0 * p->elem(), p->prec,
                                 dre, dim, c, scale, p->stream);
        if (host[b].empty()) host[b].resize(2 * (size_t)chunk);
        double *hre = host[b].data(), *him = hre + chunk;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(hre, dre, (size_t)c * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(him, dim, (size_t)c * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
        if (e == cudaSuccess) {
            wre[b] = chain(wre[b ^ 1], fr.f, hre, c);
            wim[b] = chain(wim[b ^ 1], fi.f, him, c);
        }
    }
    for (int b = 0; b < 2; ++b) {
        if (wre[b].valid()) ok = wre[b].get() && ok;
        if (wim[b].valid()) ok = wim[b].get() && ok;
    }
    if (e != cudaSuccess)
        return set_error(WSG_ERR_CUDA, "wsg_plan_dump_cube: %s", cudaGetErrorString(e));
    if (!ok) return set_error(WSG_ERR_IO, "write to %s / %s failed", real_path, img_path);
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
    auto im_ok = std::async(std::launch::async, [&]() {
        return fwrite(image_imag, sizeof(double), (size_t)npix, fi.f) == (size_t)npix;
    });
    const bool re_ok = fwrite(image_real, sizeof(double), (size_t)npix, fr.f) == (size_t)npix;
    if (!im_ok.get()) return set_error(WSG_ERR_IO, "write to %s failed", img_path);
    if (!re_ok) return set_error(WSG_ERR_IO, "write to %s failed", real_path);
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
