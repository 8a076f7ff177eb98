// kcna_io.cu - files in and out of the context.
//
// kcna_upload_lshkit reads an lshkit file (u32 header {4, rows, cols}, then
// the rows; the row count follows from the file size, as Matrix::load does,
// src/kgraph-data.h:161-177, 262-274) straight into device memory: the file
// is mapped, and chunks of 64 MiB are copied into one of two pinned staging
// buffers and sent to the device with cudaMemcpy2DAsync (rows padded to the
// device pitch), so that the page-in of one chunk overlaps the transfer of the
// previous one.  The reference loads the whole file into host memory first
// (Matrix::load_lshkit) and reads it from there.
//
// kcna_write_nsg_async snapshots the graph (one device-to-host copy) and
// writes the NSG file (SaveNsg's layout, src/kgraph.cpp:1704-1724: u32 width,
// u32 ep, per node u32 GK + GK u32 ids) on a host thread, so that the caller
// can go on (the next layer, the next index) while the file is written;
// kcna_wait_writes joins it and reports its outcome.  kcna_write_nsg is the
// two in one call.
#include <fcntl.h>
#include <stdio.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "kcna_internal.h"

namespace {

constexpr size_t IO_CHUNK = 64ull << 20; // bytes of file rows per staging buffer

struct MappedFile {
    int fd = -1;
    void *base = MAP_FAILED;
    size_t size = 0;
    ~MappedFile() {
        if (base != MAP_FAILED) munmap(base, size);
        if (fd >= 0) close(fd);
    }
};

} // namespace

extern "C" {

kcna_status kcna_upload_lshkit(kcna_ctx *c, const char *path) {
    if (!c) return KCNA_E_ARG;
    if (!path) return kcna_fail(c, KCNA_E_ARG, "upload_lshkit: null path");
    MappedFile f;
    f.fd = open(path, O_RDONLY);
    struct stat sb;
    if (f.fd < 0 || fstat(f.fd, &sb) != 0) return kcna_fail(c, KCNA_E_IO, std::string("upload_lshkit: cannot open ") + path);
    f.size = (size_t)sb.st_size;
    if (f.size < 12) return kcna_fail(c, KCNA_E_IO, std::string("upload_lshkit: no lshkit header in ") + path);
    f.base = mmap(nullptr, f.size, PROT_READ, MAP_PRIVATE, f.fd, 0);
    if (f.base == MAP_FAILED) return kcna_fail(c, KCNA_E_IO, std::string("upload_lshkit: cannot map ") + path);
    madvise(f.base, f.size, MADV_SEQUENTIAL);
    uint32_t h[3];
    memcpy(h, f.base, sizeof h);
    if (h[0] != 4 || h[2] == 0)
        return kcna_fail(c, KCNA_E_IO, std::string("upload_lshkit: not a float lshkit file: ") + path);
    const uint32_t d = h[2];
    const uint64_t row_bytes = (uint64_t)d * 4, n64 = (f.size - 12) / row_bytes;
    if (n64 > KCNA_MAX_ID) return kcna_fail(c, KCNA_E_ARG, "upload_lshkit: too many rows");
    const uint32_t n = (uint32_t)n64;
    KCNA_TRY(kcna_rows_reset(c, n, d));
    const uint64_t per = std::max<uint64_t>(1, IO_CHUNK / row_bytes); // rows per chunk
    void *stage[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    kcna_status s = KCNA_OK;
    for (int b = 0; b < 2 && s == KCNA_OK; ++b) {
        s = kcna_cuda_check(c, cudaHostAlloc(&stage[b], per * row_bytes, cudaHostAllocDefault), "pinned staging");
        if (s == KCNA_OK) s = kcna_cuda_check(c, cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming), "event");
    }
    const unsigned char *rows = static_cast<const unsigned char *>(f.base) + 12;
    uint64_t k = 0;
    for (uint64_t i0 = 0; s == KCNA_OK && i0 < n; i0 += per, ++k) {
        const int b = (int)(k & 1);
        const uint64_t m = std::min<uint64_t>(per, n - i0);
        if (k >= 2) s = kcna_cuda_check(c, cudaEventSynchronize(done[b]), "staging wait");
        if (s != KCNA_OK) break;
        memcpy(stage[b], rows + i0 * row_bytes, m * row_bytes); // pages the chunk in
        s = kcna_cuda_check(c, cudaMemcpy2DAsync(c->X + i0 * c->ld, (size_t)c->ld * 4, stage[b], row_bytes, row_bytes, m,
                                                 cudaMemcpyHostToDevice, c->stream),
                            "upload copy");
        if (s == KCNA_OK) s = kcna_cuda_check(c, cudaEventRecord(done[b], c->stream), "event record");
    }
    const kcna_status w = kcna_cuda_check(c, cudaStreamSynchronize(c->stream), "upload sync");
    if (s == KCNA_OK) s = w;
    for (int b = 0; b < 2; ++b) {
        if (stage[b]) cudaFreeHost(stage[b]);
        if (done[b]) cudaEventDestroy(done[b]);
    }
    return s;
}

kcna_status kcna_wait_writes(kcna_ctx *c) {
    if (!c) return KCNA_E_ARG;
    if (c->writer.joinable()) c->writer.join();
    const kcna_status s = c->writer_status;
    c->writer_status = KCNA_OK;
    if (s != KCNA_OK) return kcna_fail(c, s, c->writer_err);
    return KCNA_OK;
}

kcna_status kcna_write_nsg_async(kcna_ctx *c, const char *path) {
    if (!c || !c->has_graph) return kcna_fail(c, KCNA_E_STATE, "write_nsg: no graph");
    if (!path) return kcna_fail(c, KCNA_E_ARG, "write_nsg: null path");
    KCNA_TRY(kcna_wait_writes(c)); // one write in flight
    std::vector<uint32_t> ids((size_t)c->n * c->W), deg(c->n);
    uint32_t ep = 0, W = 0;
    KCNA_TRY(kcna_get_graph(c, ids.data(), deg.data(), &ep, &W));
    std::string file(path);
    c->writer = std::thread([c, file, ids = std::move(ids), deg = std::move(deg), ep, W]() {
        uint32_t width = 0;
        for (uint32_t d : deg) width = std::max(width, d);
        FILE *f = fopen(file.c_str(), "wb");
        if (!f) {
            c->writer_status = KCNA_E_IO;
            c->writer_err = "write_nsg: cannot open " + file;
            return;
        }
        std::vector<char> buf(1u << 22);
        setvbuf(f, buf.data(), _IOFBF, buf.size());
        bool ok = fwrite(&width, 4, 1, f) == 1 && fwrite(&ep, 4, 1, f) == 1;
        for (size_t i = 0; ok && i < deg.size(); ++i) {
            const uint32_t gk = std::min(deg[i], W);
            ok = fwrite(&gk, 4, 1, f) == 1 && (gk == 0 || fwrite(ids.data() + i * W, 4, gk, f) == gk);
        }
        ok = (fclose(f) == 0) && ok;
        if (!ok) {
            c->writer_status = KCNA_E_IO;
            c->writer_err = "write_nsg: write failed for " + file;
        }
    });
    return KCNA_OK;
}

kcna_status kcna_write_nsg(kcna_ctx *c, const char *path) {
    KCNA_TRY(kcna_write_nsg_async(c, path));
    return kcna_wait_writes(c);
}

} // extern "C"
