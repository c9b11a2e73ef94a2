// MRC image-stack I/O (reference AREC3D/AREC3D/arecImageIO.cpp:10-173 and the
// distributed forms of arecImageIO_mpi.cpp:7-524).
//
// The file format is the reference's: a 1024-byte header (MRCheader,
// arecImageIO.h:12-63: nx, ny, nz, mode, ... , 10 labels of 80 characters)
// followed by nz images of ny rows of nx values, x fastest, host byte order.
// Modes read: 1 and 6 as signed 16-bit integers (the reference reads both
// through `short`), 2 as float32; written: mode 2.
//
// Device path: a read streams the requested part of the file through two
// pinned host buffers (fread into one while the other is copied to the GPU)
// and converts 16-bit data to float on the device; a write computes the
// header's min / max / mean on the device (FP64 mean) and streams the data back
// the same way.  The part read is the reference's distribution of a stack over
// `nranks` ranks: by Z (arecReadImageDistbyZ: a contiguous range of images) or
// by Y (arecReadImageDistbyY: a contiguous range of rows of every image).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "arec_compat.h"
#include "arec_internal.cuh"

namespace arecgb {

const char *last_error();

struct MrcHeader {
    int nx, ny, nz, mode;
    int nxstart, nystart, nzstart;
    int mx, my, mz;
    float xlen, ylen, zlen;
    float alpha, beta, gamma;
    int mapc, mapr, maps;
    float amin, amax, amean;
    int ispg, nsymbt;
    int user[25];
    float xorigin, yorigin, zorigin;
    char map[4];
    int machinestamp;
    float rms;
    int nlabels;
    char labels[10][80];
};
static_assert(sizeof(MrcHeader) == 1024, "MRC header is 1024 bytes");

namespace {

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

int mrc_open(const char *fname, const char *how, File &fh) {
    fh.f = fopen(fname, how);
    if (!fh.f) {
        set_error(std::string("failed to open ") + fname);
        return ARECGB_ERR_ARG;
    }
    return 0;
}

int read_header(FILE *f, const char *fname, MrcHeader &h) {
    if (fread(&h, sizeof(h), 1, f) != 1) {
        set_error(std::string("failed to read an MRC header from ") + fname);
        return ARECGB_ERR_ARG;
    }
    if (h.nx < 0 || h.ny < 0 || h.nz < 0) {
        set_error(std::string("negative MRC dimensions in ") + fname);
        return ARECGB_ERR_ARG;
    }
    return 0;
}

// The reference's split of n items over nranks: the first n % nranks ranks
// take one more (arecImageIO_mpi.cpp:46-48, 169-178).
void split(int n, int rank, int nranks, int &off, int &cnt) {
    const int base = n / nranks, rem = n % nranks;
    cnt = base + (rank < rem ? 1 : 0);
    off = rank * base + (rank < rem ? rank : rem);
}

__global__ void k_i16_to_f32(const short *__restrict__ in, float *__restrict__ out, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// min / max and FP64 sum per block, then one block combines them in order.
constexpr int kStatBlocks = 1024, kStatThreads = 256;

__global__ void k_stats_partial(const float *__restrict__ x, size_t n, double *__restrict__ part) {
    __shared__ double smin[kStatThreads], smax[kStatThreads], ssum[kStatThreads];
    double mn = 1.0e20, mx = -1.0e20, s = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
        s += v;
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    ssum[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = smin[0];
        part[3 * blockIdx.x + 1] = smax[0];
        part[3 * blockIdx.x + 2] = ssum[0];
    }
}

__global__ void k_stats_final(const double *part, int nb, double *out) {
    if (threadIdx.x || blockIdx.x) return;
    double mn = 1.0e20, mx = -1.0e20, s = 0.0;
    for (int b = 0; b < nb; b++) {
        mn = fmin(mn, part[3 * b]);
        mx = fmax(mx, part[3 * b + 1]);
        s += part[3 * b + 2];
    }
    out[0] = mn;
    out[1] = mx;
    out[2] = s;
}

constexpr size_t kChunkBytes = size_t(32) << 20;  // per pinned staging buffer

struct Pinned {
    void *p[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    ~Pinned() {
        for (int i = 0; i < 2; i++) {
            if (ev[i]) {
                cudaEventSynchronize(ev[i]);
                cudaEventDestroy(ev[i]);
            }
            if (p[i]) cudaFreeHost(p[i]);
        }
    }
    int init() {
        for (int i = 0; i < 2; i++) {
            ARECGB_CUDA(cudaMallocHost(&p[i], kChunkBytes));
            ARECGB_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        }
        return 0;
    }
};

}  // namespace

void mrc_header_defaults(MrcHeader &h, int nx, int ny, int nz) {
    // the fields arecWriteImage sets (arecImageIO.cpp:98-155); the ones it
    // leaves unset (machinestamp, labels) are written as zero
    memset(&h, 0, sizeof(h));
    h.nx = nx;
    h.ny = ny;
    h.nz = nz;
    h.mode = 2;
    h.mx = nx;
    h.my = ny;
    h.mz = nz;
    h.xlen = h.ylen = h.zlen = 1;
    h.alpha = h.beta = h.gamma = 90.0f;
    h.mapc = 1;
    h.mapr = 2;
    h.maps = 3;
    for (int i = 0; i < 25; i++) h.user[i] = ' ';
    h.user[24] = '\0';
    h.map[0] = 'M';
    h.map[1] = 'A';
    h.map[2] = 'P';
    h.map[3] = '\0';
    h.rms = 1.0f;
}

int mrc_read_header(const char *fname, int *nx, int *ny, int *nz, int *mode) {
    File fh;
    if (int rc = mrc_open(fname, "rb", fh)) return rc;
    MrcHeader h;
    if (int rc = read_header(fh.f, fname, h)) return rc;
    if (nx) *nx = h.nx;
    if (ny) *ny = h.ny;
    if (nz) *nz = h.nz;
    if (mode) *mode = h.mode;
    return 0;
}

// Read this rank's part of a stack into device memory [nz_loc][ny_loc][nx].
int mrc_read_device(const char *fname, int rank, int nranks, int by_y, float *d_out,
                    size_t cap_floats, int *nx_out, int *ny_out, int *nz_out, cudaStream_t st) {
    if (nranks < 1 || rank < 0 || rank >= nranks) {
        set_error("mrc_read: rank must be in [0, nranks)");
        return ARECGB_ERR_ARG;
    }
    File fh;
    if (int rc = mrc_open(fname, "rb", fh)) return rc;
    MrcHeader h;
    if (int rc = read_header(fh.f, fname, h)) return rc;
    const int mode = h.mode;
    if (mode != 1 && mode != 2 && mode != 6) {
        set_error("mrc_read: invalid mrc mode " + std::to_string(mode));
        return ARECGB_ERR_ARG;
    }
    const size_t es = mode == 2 ? 4 : 2;
    int z0 = 0, nzl = h.nz, y0 = 0, nyl = h.ny;
    if (by_y)
        split(h.ny, rank, nranks, y0, nyl);
    else
        split(h.nz, rank, nranks, z0, nzl);
    if (nx_out) *nx_out = h.nx;
    if (ny_out) *ny_out = nyl;
    if (nz_out) *nz_out = nzl;
    const size_t piece = (size_t)nyl * h.nx;  // values per image read
    const size_t total = piece * nzl;
    if (!d_out) return 0;  // size query
    if (total > cap_floats) {
        set_error("mrc_read: output holds " + std::to_string(cap_floats) + " floats, " +
                  std::to_string(total) + " needed");
        return ARECGB_ERR_ARG;
    }
    if (total == 0) return 0;
    Pinned pin;
    if (int rc = pin.init()) return rc;
    void *d_raw = nullptr;  // 16-bit staging on the device
    if (es == 2) ARECGB_CUDA(cudaMallocAsync(&d_raw, 2 * kChunkBytes, st));
    // images per chunk: whole pieces, at least one (a piece larger than the
    // chunk is read in row ranges)
    const size_t piece_bytes = piece * es;
    const size_t row_bytes = (size_t)h.nx * es;
    int rc = 0;
    size_t done = 0;  // values delivered
    int k = 0;
    const long long img_bytes = (long long)h.ny * h.nx * (long long)es;
    for (int z = 0; z < nzl && !rc;) {
        // a chunk: images z.. (or part of image z when one piece is too big)
        size_t bytes = 0;
        int zc = 0;
        size_t r0 = 0, nr = 0;  // row range within image z when splitting an image
        if (piece_bytes <= kChunkBytes) {
            zc = (int)std::min<size_t>((size_t)(nzl - z), kChunkBytes / piece_bytes);
            bytes = (size_t)zc * piece_bytes;
        } else {
            const size_t rows_per = std::max<size_t>(1, kChunkBytes / row_bytes);
            const size_t got = (done - (size_t)z * piece) / h.nx;  // rows of image z done
            r0 = got;
            nr = std::min<size_t>((size_t)nyl - got, rows_per);
            bytes = nr * row_bytes;
        }
        const int b = k & 1;
        if (cudaEventSynchronize(pin.ev[b]) != cudaSuccess) {  // buffer free again
            set_error("mrc_read: staging event failed");
            rc = ARECGB_ERR_CUDA_BASE;
            break;
        }
        char *hb = (char *)pin.p[b];
        if (zc > 0) {
            for (int j = 0; j < zc && !rc; j++) {
                const long long off = (long long)sizeof(MrcHeader) + (long long)(z0 + z + j) * img_bytes +
                                      (long long)y0 * (long long)row_bytes;
                if (fseeko(fh.f, (off_t)off, SEEK_SET) != 0 ||
                    fread(hb + (size_t)j * piece_bytes, 1, piece_bytes, fh.f) != piece_bytes) {
                    set_error(std::string("mrc_read: failed to read ") + fname);
                    rc = ARECGB_ERR_ARG;
                }
            }
        } else {
            const long long off = (long long)sizeof(MrcHeader) + (long long)(z0 + z) * img_bytes +
                                  (long long)(y0 + r0) * (long long)row_bytes;
            if (fseeko(fh.f, (off_t)off, SEEK_SET) != 0 || fread(hb, 1, bytes, fh.f) != bytes) {
                set_error(std::string("mrc_read: failed to read ") + fname);
                rc = ARECGB_ERR_ARG;
            }
        }
        if (rc) break;
        const size_t nval = bytes / es;
        cudaError_t e;
        if (es == 4) {
            e = cudaMemcpyAsync(d_out + done, hb, bytes, cudaMemcpyHostToDevice, st);
        } else {
            short *dr = (short *)((char *)d_raw + (size_t)b * kChunkBytes);
            e = cudaMemcpyAsync(dr, hb, bytes, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) {
                const int blocks = (int)std::min<size_t>(1024, (nval + 255) / 256);
                k_i16_to_f32<<<blocks, 256, 0, st>>>(dr, d_out + done, nval);
                count_launches(1);
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(pin.ev[b], st);
        if (e != cudaSuccess) {
            set_error(std::string("mrc_read: ") + cudaGetErrorString(e));
            rc = cuda_status(e);
            break;
        }
        done += nval;
        k++;
        if (zc > 0)
            z += zc;
        else if (r0 + nr == (size_t)nyl)
            z++;
    }
    if (d_raw) cudaFreeAsync(d_raw, st);
    if (!rc) ARECGB_CUDA(cudaStreamSynchronize(st));
    return rc;
}

// Write a device stack [nz][ny][nx] as a mode-2 MRC file with the header
// arecWriteImage writes (min, max, mean of the data).
int mrc_write_device(const char *fname, const float *d_in, int nz, int ny, int nx,
                     cudaStream_t st) {
    if (nx < 0 || ny < 0 || nz < 0) {
        set_error("mrc_write: negative dimensions");
        return ARECGB_ERR_ARG;
    }
    const size_t n = (size_t)nx * ny * nz;
    MrcHeader h;
    mrc_header_defaults(h, nx, ny, nz);
    double stats[3] = {1.0e20, -1.0e20, 0.0};
    if (n) {
        double *d_part = nullptr;
        ARECGB_CUDA(cudaMallocAsync(&d_part, sizeof(double) * (3 * kStatBlocks + 3), st));
        k_stats_partial<<<kStatBlocks, kStatThreads, 0, st>>>(d_in, n, d_part);
        k_stats_final<<<1, 32, 0, st>>>(d_part, kStatBlocks, d_part + 3 * kStatBlocks);
        count_launches(2);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(stats, d_part + 3 * kStatBlocks, sizeof(stats),
                                cudaMemcpyDeviceToHost, st);
        cudaFreeAsync(d_part, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_error(std::string("mrc_write: ") + cudaGetErrorString(e));
            return cuda_status(e);
        }
    }
    h.amin = (float)stats[0];
    h.amax = (float)stats[1];
    h.amean = (float)(stats[2] / (float)n);
    File fh;
    if (int rc = mrc_open(fname, "wb", fh)) return rc;
    if (fwrite(&h, sizeof(h), 1, fh.f) != 1) {
        set_error("failed to write an MRC header");
        return ARECGB_ERR_ARG;
    }
    if (n == 0) return 0;
    Pinned pin;
    if (int rc = pin.init()) return rc;
    const size_t per = kChunkBytes / sizeof(float);
    const size_t nchunks = (n + per - 1) / per;
    // copy chunk k+1 back while chunk k is written
    auto issue = [&](size_t k) -> cudaError_t {
        const size_t o = k * per, m = std::min(per, n - o);
        cudaError_t e = cudaMemcpyAsync(pin.p[k & 1], d_in + o, m * sizeof(float),
                                        cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaEventRecord(pin.ev[k & 1], st);
        return e;
    };
    cudaError_t e = issue(0);
    for (size_t k = 0; k < nchunks && e == cudaSuccess; k++) {
        e = cudaEventSynchronize(pin.ev[k & 1]);
        if (e == cudaSuccess && k + 1 < nchunks) e = issue(k + 1);
        if (e != cudaSuccess) break;
        const size_t o = k * per, m = std::min(per, n - o);
        if (fwrite(pin.p[k & 1], sizeof(float), m, fh.f) != m) {
            set_error("failed to write MRC data");
            ARECGB_CUDA(cudaStreamSynchronize(st));
            return ARECGB_ERR_ARG;
        }
    }
    if (e != cudaSuccess) {
        set_error(std::string("mrc_write: ") + cudaGetErrorString(e));
        return cuda_status(e);
    }
    return 0;
}

}  // namespace arecgb

// ===========================================================================
// C ABI and the reference's host entry points.

using namespace arecgb;

namespace {

// Host read of this rank's part (the reference's own arithmetic: 16-bit values
// converted with (float)short).
int read_stack_host(const char *who, const char *fname, int rank, int nranks, int by_y,
                    arecImage *image) {
    image->data = nullptr;
    File fh;
    if (int rc = mrc_open(fname, "rb", fh)) return rc;
    MrcHeader h;
    if (int rc = read_header(fh.f, fname, h)) return rc;
    if (h.mode != 1 && h.mode != 2 && h.mode != 6) {
        set_error(std::string(who) + ": invalid mrc mode: " + std::to_string(h.mode));
        return ARECGB_ERR_ARG;
    }
    int z0 = 0, nzl = h.nz, y0 = 0, nyl = h.ny;
    if (by_y)
        split(h.ny, rank, nranks, y0, nyl);
    else
        split(h.nz, rank, nranks, z0, nzl);
    const size_t es = h.mode == 2 ? 4 : 2, piece = (size_t)nyl * h.nx;
    float *data = (float *)malloc(std::max<size_t>(1, piece * nzl) * sizeof(float));
    std::vector<short> sbuf(h.mode == 2 ? 0 : piece);
    if (!data) {
        set_error(std::string(who) + ": failed to allocate image data");
        return ARECGB_ERR_NOMEM;
    }
    const long long img_bytes = (long long)h.ny * h.nx * (long long)es;
    for (int z = 0; z < nzl; z++) {
        const long long off = (long long)sizeof(MrcHeader) + (long long)(z0 + z) * img_bytes +
                              (long long)y0 * h.nx * (long long)es;
        float *dst = data + (size_t)z * piece;
        bool ok = fseeko(fh.f, (off_t)off, SEEK_SET) == 0;
        if (ok && es == 4) {
            ok = fread(dst, sizeof(float), piece, fh.f) == piece;
        } else if (ok) {
            ok = fread(sbuf.data(), sizeof(short), piece, fh.f) == piece;
            for (size_t i = 0; ok && i < piece; i++) dst[i] = (float)sbuf[i];
        }
        if (!ok) {
            free(data);
            set_error(std::string(who) + ": failed to read " + fname);
            return ARECGB_ERR_ARG;
        }
    }
    image->data = data;
    image->nx = h.nx;
    image->ny = nyl;
    image->nz = nzl;
    image->cord = nullptr;
    image->is_cyl = 0;
    return 0;
}

// Host write with the header statistics of the reference entry point:
// arecWriteImage sums the mean in double, arecWriteImageMerge{Y,Z} in float.
int write_stack_host(const char *fname, const arecImage &im, bool float_mean) {
    const size_t n = (size_t)im.nx * im.ny * im.nz;
    MrcHeader h;
    mrc_header_defaults(h, im.nx, im.ny, im.nz);
    if (float_mean) {
        float amin = 1.0e20f, amax = -1.0e20f, mean = 0.0f;
        for (size_t i = 0; i < n; i++) {
            if (im.data[i] > amax) amax = im.data[i];
            if (im.data[i] < amin) amin = im.data[i];
            mean = mean + im.data[i];
        }
        h.amean = mean / (float)(im.nx * im.ny * im.nz);
        h.amax = amax;
        h.amin = amin;
    } else {
        double amin = 1.0e20, amax = -1.0e20, mean = 0.0;
        for (size_t i = 0; i < n; i++) {
            if (im.data[i] > amax) amax = im.data[i];
            if (im.data[i] < amin) amin = im.data[i];
            mean = mean + im.data[i];
        }
        mean = mean / (float)(im.nx * im.ny * im.nz);
        h.amin = (float)amin;
        h.amax = (float)amax;
        h.amean = (float)mean;
    }
    File fh;
    if (int rc = mrc_open(fname, "wb", fh)) return rc;
    if (fwrite(&h, sizeof(h), 1, fh.f) != 1) {
        set_error("failed to write an MRC header");
        return ARECGB_ERR_ARG;
    }
    if (n && fwrite(im.data, sizeof(float), n, fh.f) != n) {
        set_error("failed to write MRC data");
        return ARECGB_ERR_ARG;
    }
    return 0;
}

bool quiet_io() {
    const char *q = getenv("ARECGB_QUIET");
    return q && q[0] && q[0] != '0';
}

}  // namespace

extern "C" {

int arecgb_mrc_read_header(const char *fname, int *nx, int *ny, int *nz, int *mode) {
    return mrc_read_header(fname, nx, ny, nz, mode);
}

int arecgb_mrc_read_device(const char *fname, int rank, int nranks, int by_y, float *d_out,
                           size_t cap_floats, int *nx, int *ny_loc, int *nz_loc, void *stream) {
    return mrc_read_device(fname, rank, nranks, by_y, d_out, cap_floats, nx, ny_loc, nz_loc,
                           (cudaStream_t)stream);
}

int arecgb_mrc_write_device(const char *fname, const float *d_in, int nz, int ny, int nx,
                            void *stream) {
    return mrc_write_device(fname, d_in, nz, ny, nx, (cudaStream_t)stream);
}

// arecReadImageHeader (AREC3D/AREC3D/arecImageIO.cpp:10-29).
int arecgb_arecReadImageHeader(char *fname, int *nx, int *ny, int *nz) {
    if (mrc_read_header(fname, nx, ny, nz, nullptr)) {
        if (!quiet_io()) fprintf(stderr, "failed to open %s\n", fname);
        return -1;
    }
    return 0;
}

// arecReadImage (AREC3D/AREC3D/arecImageIO.cpp:31-82): the whole stack.
int arecgb_arecReadImage(char *fname, arecImage *image) {
    if (read_stack_host("arecReadImage", fname, 0, 1, 0, image)) {
        if (!quiet_io()) fprintf(stderr, "arecReadImage: %s\n", last_error());
        return -1;
    }
    return 0;
}

// arecWriteImage (AREC3D/AREC3D/arecImageIO.cpp:84-173).
int arecgb_arecWriteImage(char *fname, arecImage image) {
    if (write_stack_host(fname, image, false)) {
        if (!quiet_io()) fprintf(stderr, "%s\n", last_error());
        return -1;
    }
    return 0;
}

// arecReadImageDistbyZ / DistbyY (AREC3D/AREC3D/arecImageIO_mpi.cpp:7-260) and
// arecWriteImageMergeY / MergeZ (:262-524) for the single rank this library
// runs as: the whole stack.  Failures print and leave image->data NULL where
// the reference calls MPI_Abort.
void arecgb_arecReadImageDistbyZ(MPI_Comm, const char *fname, arecImage *image) {
    if (read_stack_host("arecReadImageDistbyZ", fname, 0, 1, 0, image) && !quiet_io())
        fprintf(stderr, "%s\n", last_error());
}

void arecgb_arecReadImageDistbyY(MPI_Comm, const char *fname, arecImage *image) {
    if (read_stack_host("arecReadImageDistbyY", fname, 0, 1, 1, image) && !quiet_io())
        fprintf(stderr, "%s\n", last_error());
}

void arecgb_arecWriteImageMergeY(MPI_Comm, const char *fname, arecImage image) {
    if (write_stack_host(fname, image, true) && !quiet_io())
        fprintf(stderr, "%s\n", last_error());
}

void arecgb_arecWriteImageMergeZ(MPI_Comm, const char *fname, arecImage image) {
    if (write_stack_host(fname, image, true) && !quiet_io())
        fprintf(stderr, "%s\n", last_error());
}

}  // extern "C"

// The reference's C++ names (arecImageIO.h:65-67, arecImageIO_mpi.h).
int arecReadImageHeader(char *f, int *nx, int *ny, int *nz) { return arecgb_arecReadImageHeader(f, nx, ny, nz); }
int arecReadImage(char *f, arecImage *i) { return arecgb_arecReadImage(f, i); }
int arecWriteImage(char *f, arecImage i) { return arecgb_arecWriteImage(f, i); }
void arecReadImageDistbyZ(MPI_Comm c, const char *f, arecImage *i) { arecgb_arecReadImageDistbyZ(c, f, i); }
void arecReadImageDistbyY(MPI_Comm c, const char *f, arecImage *i) { arecgb_arecReadImageDistbyY(c, f, i); }
void arecWriteImageMergeY(MPI_Comm c, const char *f, arecImage i) { arecgb_arecWriteImageMergeY(c, f, i); }
void arecWriteImageMergeZ(MPI_Comm c, const char *f, arecImage i) { arecgb_arecWriteImageMergeZ(c, f, i); }
