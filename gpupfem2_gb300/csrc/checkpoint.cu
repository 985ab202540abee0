// checkpoint.cu - the checkpoint file format shared by particles and flow engines.
//
// The reference keeps no restart files; a long run of its drivers starts from the seed
// every time.  Layout (little-endian, as the host writes it):
//   "PF2CKPT\0"  u32 version  u32 kind
//   then per section: char tag[8] (zero padded)  u64 length  payload
// Sections come in the order the writer emits them; the reader names what it expects.
#include <cstring>

#include "common.cuh"
#include "internal.cuh"

namespace pf2 {

namespace {
constexpr char kMagic[8] = { 'P', 'F', '2', 'C', 'K', 'P', 'T', '\0' };
constexpr uint32_t kVersion = 1;

// a section tag: up to 8 characters, NUL-padded (not NUL-terminated at 8)
void tag8(const char* tag, char out[8]) {
    memset(out, 0, 8);
    for (int i = 0; i < 8 && tag[i]; ++i) out[i] = tag[i];
}
}  // namespace

CkptFile::~CkptFile() {
    if (f_) fclose(f_);
}

pf2_status CkptFile::open_write(const char* path, CkptKind kind) {
    PF2_REQUIRE(path, PF2_BAD_INPUT, "null path");
    f_ = fopen(path, "wb");
    PF2_REQUIRE(f_, PF2_IO_ERROR, "cannot open %s for writing", path);
    wr_ = true;
    path_ = path;
    const uint32_t h[2] = { kVersion, (uint32_t)kind };
    PF2_REQUIRE(fwrite(kMagic, 1, 8, f_) == 8 && fwrite(h, sizeof(h), 1, f_) == 1, PF2_IO_ERROR,
                "write error on %s", path);
    return PF2_OK;
}

pf2_status CkptFile::open_read(const char* path, CkptKind kind) {
    PF2_REQUIRE(path, PF2_BAD_INPUT, "null path");
    f_ = fopen(path, "rb");
    PF2_REQUIRE(f_, PF2_IO_ERROR, "cannot open %s", path);
    wr_ = false;
    path_ = path;
    char m[8];
    uint32_t h[2];
    PF2_REQUIRE(fread(m, 1, 8, f_) == 8 && memcmp(m, kMagic, 8) == 0, PF2_BAD_INPUT, "%s is not a checkpoint", path);
    PF2_REQUIRE(fread(h, sizeof(h), 1, f_) == 1, PF2_BAD_INPUT, "%s: truncated header", path);
    PF2_REQUIRE(h[0] == kVersion, PF2_BAD_INPUT, "%s: format version %u, this library reads %u", path, h[0], kVersion);
    PF2_REQUIRE(h[1] == (uint32_t)kind, PF2_BAD_INPUT, "%s holds object kind %u, expected %u", path, h[1],
                (uint32_t)kind);
    return PF2_OK;
}

pf2_status CkptFile::close() {
    PF2_REQUIRE(f_, PF2_BAD_INPUT, "checkpoint not open");
    FILE* f = f_;
    f_ = nullptr;
    if (wr_) {
        const bool ok = fflush(f) == 0 && !ferror(f);
        const bool closed = fclose(f) == 0;
        PF2_REQUIRE(ok && closed, PF2_IO_ERROR, "write error on %s", path_.c_str());
        return PF2_OK;
    }
    const int c = fgetc(f);
    fclose(f);
    PF2_REQUIRE(c == EOF, PF2_BAD_INPUT, "%s: data after the last section", path_.c_str());
    return PF2_OK;
}

pf2_status CkptFile::header(const char* tag, size_t bytes) {
    char t[8];
    tag8(tag, t);
    const uint64_t len = bytes;
    if (wr_) {
        PF2_REQUIRE(fwrite(t, 1, 8, f_) == 8 && fwrite(&len, sizeof(len), 1, f_) == 1, PF2_IO_ERROR,
                    "write error on %s", path_.c_str());
        return PF2_OK;
    }
    char rt[9] = { 0 };
    uint64_t rlen = 0;
    PF2_REQUIRE(fread(rt, 1, 8, f_) == 8 && fread(&rlen, sizeof(rlen), 1, f_) == 1, PF2_BAD_INPUT,
                "%s: truncated before section '%.8s'", path_.c_str(), t);
    PF2_REQUIRE(memcmp(rt, t, 8) == 0, PF2_BAD_INPUT, "%s: section '%s' where '%.8s' was expected", path_.c_str(), rt,
                t);
    PF2_REQUIRE(rlen == len, PF2_BAD_INPUT, "%s: section '%.8s' holds %llu bytes, expected %llu", path_.c_str(), t,
                (unsigned long long)rlen, (unsigned long long)len);
    return PF2_OK;
}

pf2_status CkptFile::host(const char* tag, void* p, size_t bytes) {
    PF2_REQUIRE(f_, PF2_BAD_INPUT, "checkpoint not open");
    PF2_TRY(header(tag, bytes));
    if (bytes == 0) return PF2_OK;
    if (wr_) {
        PF2_REQUIRE(fwrite(p, 1, bytes, f_) == bytes, PF2_IO_ERROR, "write error on %s", path_.c_str());
    } else {
        PF2_REQUIRE(fread(p, 1, bytes, f_) == bytes, PF2_BAD_INPUT, "%s: section '%s' truncated", path_.c_str(), tag);
    }
    return PF2_OK;
}

pf2_status CkptFile::device(const char* tag, void* d, size_t bytes, cudaStream_t st) {
    stage_.resize(bytes);
    if (wr_ && bytes) {
        PF2_CUDA(cudaMemcpyAsync(stage_.data(), d, bytes, cudaMemcpyDeviceToHost, st));
        PF2_CUDA(cudaStreamSynchronize(st));
    }
    PF2_TRY(host(tag, stage_.data(), bytes));
    if (!wr_ && bytes) {
        PF2_CUDA(cudaMemcpyAsync(d, stage_.data(), bytes, cudaMemcpyHostToDevice, st));
        PF2_CUDA(cudaStreamSynchronize(st));
    }
    return PF2_OK;
}

}  // namespace pf2
