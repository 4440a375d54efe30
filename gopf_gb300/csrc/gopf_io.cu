// gopf_io.cu -- field files in the reference's raw format (pf/fileIO.go).
//
// Float64IO.SaveFields / SaveFloat64 (pf/fileIO.go:45-97) write the real part
// of a field as raw big-endian float64 values in node order; LoadFloat64 reads
// them back.  Here the field goes from the device's spectral state to real
// space (x pass), to FP64, and through the byte swap on the GPU, lands in a
// pinned staging buffer owned by the context, and is written by a host thread.
// With async set, gopf_save_float64 returns once the copy is queued: the
// device keeps stepping while the file is written, and the next save (or
// gopf_io_wait) waits for the writer.  gopf_load_float64 is the restart path
// (LoadFloat64 followed by an upload).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>

#include "gopf_ctx.h"

int gopf_fail(gopf_ctx *ctx, int code, const std::string &msg);
int gopf_field_to_real(gopf_ctx *ctx, int f, void *dst);

struct gopf_io_state {
    double *h_stage = nullptr; // pinned, N doubles
    size_t n = 0;
    std::thread writer;
    int last_rc = GOPF_OK;
    std::string last_err;
};

namespace {

// real field (FP32 or FP64) -> big-endian FP64 bytes
template <typename R>
__global__ void k_to_be64(const R *__restrict__ in, unsigned long long *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = (double)in[i];
        unsigned long long b = (unsigned long long)__double_as_longlong(v);
        b = ((b & 0x00000000FFFFFFFFull) << 32) | ((b & 0xFFFFFFFF00000000ull) >> 32);
        b = ((b & 0x0000FFFF0000FFFFull) << 16) | ((b & 0xFFFF0000FFFF0000ull) >> 16);
        b = ((b & 0x00FF00FF00FF00FFull) << 8) | ((b & 0xFF00FF00FF00FF00ull) >> 8);
        out[i] = b;
    }
}

unsigned long long bswap64(unsigned long long b)
{
    b = ((b & 0x00000000FFFFFFFFull) << 32) | ((b & 0xFFFFFFFF00000000ull) >> 32);
    b = ((b & 0x0000FFFF0000FFFFull) << 16) | ((b & 0xFFFF0000FFFF0000ull) >> 16);
    b = ((b & 0x00FF00FF00FF00FFull) << 8) | ((b & 0xFF00FF00FF00FF00ull) >> 8);
    return b;
}

int join_writer(gopf_ctx *ctx)
{
    gopf_io_state *io = ctx->io;
    if (!io) return GOPF_OK;
    if (io->writer.joinable()) io->writer.join();
    if (io->last_rc != GOPF_OK) {
        const int rc = io->last_rc;
        io->last_rc = GOPF_OK;
        return gopf_fail(ctx, rc, io->last_err);
    }
    return GOPF_OK;
}

int write_file(const std::string &path, const void *data, size_t bytes, std::string *err)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        *err = "cannot open " + path + " for writing";
        return GOPF_ERR_ARG;
    }
    const size_t w = std::fwrite(data, 1, bytes, f);
    const int c = std::fclose(f);
    if (w != bytes || c != 0) {
        *err = "short write to " + path;
        return GOPF_ERR_ARG;
    }
    return GOPF_OK;
}

} // namespace

void gopf_io_free(gopf_ctx *ctx)
{
    gopf_io_state *io = ctx->io;
    if (!io) return;
    if (io->writer.joinable()) io->writer.join();
    if (io->h_stage) cudaFreeHost(io->h_stage);
    delete io;
    ctx->io = nullptr;
}

extern "C" int gopf_io_wait(gopf_ctx *ctx)
{
    if (!ctx) return GOPF_ERR_ARG;
    return join_writer(ctx);
}

extern "C" int gopf_save_float64(gopf_ctx *ctx, int field, const char *path, int async)
{
    if (!ctx || !path) return GOPF_ERR_ARG;
    if (field < 0 || field >= std::max(ctx->nfields, 1)) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field id");
    if (!ctx->state_valid) return gopf_fail(ctx, GOPF_ERR_STATE, "field has not been uploaded");
    gopf_nvtx_scope trace("gopf_save_float64");
    int rc;
    if ((rc = join_writer(ctx))) return rc; // the staging buffer is free again
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gopf_fail(ctx, GOPF_ERR_CUDA, "cudaSetDevice");
    const size_t n = (size_t)ctx->g.N;
    if (!ctx->io) ctx->io = new gopf_io_state();
    gopf_io_state *io = ctx->io;
    if (io->n != n) {
        if (io->h_stage) cudaFreeHost(io->h_stage);
        io->h_stage = nullptr;
        if (cudaMallocHost(&io->h_stage, n * sizeof(double)) != cudaSuccess)
            return gopf_fail(ctx, GOPF_ERR_OOM, "cudaMallocHost(file staging)");
        io->n = n;
    }
    // spectral state -> real rows (d_real) -> big-endian FP64 (the staging area d_c128)
    if ((rc = gopf_field_to_real(ctx, field, ctx->d_real))) return rc;
    const unsigned blocks = (unsigned)std::min<long long>(((long long)n + 255) / 256, 152 * 16);
    unsigned long long *d_be = reinterpret_cast<unsigned long long *>(ctx->d_c128);
    if (ctx->prec == GOPF_FP32) k_to_be64<float><<<blocks, 256, 0, ctx->stream>>>((const float *)ctx->d_real, d_be, (long long)n);
    else k_to_be64<double><<<blocks, 256, 0, ctx->stream>>>((const double *)ctx->d_real, d_be, (long long)n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(io->h_stage, d_be, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaEvent_t done = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(done, ctx->stream);
    if (e != cudaSuccess) {
        if (done) cudaEventDestroy(done);
        return gopf_fail(ctx, GOPF_ERR_CUDA, std::string("save: ") + cudaGetErrorString(e));
    }
    const std::string p(path);
    auto job = [io, done, p, n]() {
        cudaError_t e2 = cudaEventSynchronize(done);
        cudaEventDestroy(done);
        if (e2 != cudaSuccess) {
            io->last_rc = GOPF_ERR_CUDA;
            io->last_err = std::string("save: ") + cudaGetErrorString(e2);
            return;
        }
        io->last_rc = write_file(p, io->h_stage, n * sizeof(double), &io->last_err);
    };
    if (async) {
        io->writer = std::thread(job);
        return GOPF_OK;
    }
    job();
    return join_writer(ctx);
}

extern "C" int gopf_load_float64(gopf_ctx *ctx, int field, const char *path)
{
    if (!ctx || !path) return GOPF_ERR_ARG;
    if (field < 0 || field >= std::max(ctx->nfields, 1)) return gopf_fail(ctx, GOPF_ERR_ARG, "bad field id");
    const size_t n = (size_t)ctx->g.N;
    FILE *f = std::fopen(path, "rb");
    if (!f) return gopf_fail(ctx, GOPF_ERR_ARG, std::string("cannot open ") + path);
    std::string buf(n * sizeof(double), '\0');
    const size_t r = std::fread(&buf[0], 1, buf.size(), f);
    const int extra = std::fgetc(f);
    std::fclose(f);
    if (r != buf.size() || extra != EOF)
        return gopf_fail(ctx, GOPF_ERR_ARG, "file size does not match the domain (expected " + std::to_string(n) +
                                                " big-endian float64 values)");
    double *vals = reinterpret_cast<double *>(&buf[0]);
    for (size_t i = 0; i < n; ++i) {
        unsigned long long b;
        std::memcpy(&b, vals + i, 8);
        b = bswap64(b);
        std::memcpy(vals + i, &b, 8);
    }
    return gopf_field_upload_real(ctx, field, vals, n);
}
