// Particle files: classic BGEO frames and numbered series of them.
//
// Reference: Dataset::Dataset (src/app/Dataset.cpp:169-227) collects the file
// names prefix + i + suffix for i = 1, 2, ... until a file is missing or i
// passes `count`, reads each with Partio::read, and Dataset::ReadFile
// (:292-306) copies the "position" of every particle into a new Frame.
// Partio's reader (vendor/partio/src/io/BGEO.cpp, readBGEO) decompresses gzip
// files (detected by their magic), checks the magic "Bgeo" and version 5,
// takes the point attribute definitions, then reads one big-endian record per
// point whose first three words are the position.
//
// Here the file is read and decompressed on the host (inflate.cpp), the point
// records go to the device as they are, and a kernel byte-swaps the three
// position words of every record into xyz, which the grid build of
// fm_scene_create takes directly.  A series keeps host threads decoding the
// frames after the one last asked for, so that an autoplay loop (the next
// frame once a march finishes, AdvancedRenderer.cpp:281-297) finds them
// ready.

#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <filesystem>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "fm_internal.cuh"
#include "fm_io.h"

namespace fm {
namespace io {

namespace {

uint32_t be32(const uint8_t* p) {
    return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | (uint32_t)p[3];
}
uint16_t be16(const uint8_t* p) { return (uint16_t)((uint32_t)p[0] << 8 | (uint32_t)p[1]); }

int fail(std::string& err, const std::string& msg) {
    err = msg;
    return -1;
}

// bytes [0, limit) of the file (the whole file when limit is 0); total = file size
int read_file(const char* path, size_t limit, std::vector<uint8_t>& out, uint64_t& total, std::string& err) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(err, std::string("cannot open '") + path + "'");
    int rc = 0;
    if (std::fseek(f, 0, SEEK_END) != 0) rc = fail(err, "cannot seek");
    const long sz = rc ? -1 : std::ftell(f);
    if (!rc && sz < 0) rc = fail(err, "cannot size the file");
    if (!rc) {
        total = (uint64_t)sz;
        const size_t want = limit && limit < (size_t)sz ? limit : (size_t)sz;
        out.resize(want);
        std::rewind(f);
        if (want && std::fread(out.data(), 1, want, f) != want) rc = fail(err, std::string("cannot read '") + path + "'");
    }
    std::fclose(f);
    return rc;
}

// The last 4 bytes of a file (a gzip member's size field), little-endian.
bool read_tail32(const char* path, uint32_t& v) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    uint8_t b[4];
    const bool ok = std::fseek(f, -4, SEEK_END) == 0 && std::fread(b, 1, 4, f) == 4;
    std::fclose(f);
    v = (uint32_t)b[0] | (uint32_t)b[1] << 8 | (uint32_t)b[2] << 16 | (uint32_t)b[3] << 24;
    return ok;
}

// A header whose point block cannot fit the file: plain files by their size,
// gzip files by the member's size field.  That field is the inflated size
// modulo 2^32, so it proves a short block only for a member that cannot
// inflate past 4 GB (DEFLATE expands at most ~1032:1: below ~4 MB
// compressed); larger gzip files are checked when they are decoded.
int check_point_block(const char* path, const BgeoFile& f, std::string& err) {
    const uint64_t need = (uint64_t)f.layout.data_offset + f.layout.points * 4ull * f.layout.words;
    if (!f.compressed) {
        if (need > f.file_bytes) return fail(err, "BGEO point data is truncated");
        return 0;
    }
    uint32_t isize = 0;
    const bool exact = 1032ull * f.file_bytes + 65536 < (1ull << 32);
    if (exact && read_tail32(path, isize) && need > isize) return fail(err, "BGEO point data is truncated");
    return 0;
}

}  // namespace

int bgeo_layout(const uint8_t* d, size_t n, bool need_points, BgeoLayout& L, std::string& err) {
    // magic, version character, then nine big-endian int32: version, points,
    // primitives, point groups, primitive groups, point / vertex / primitive /
    // detail attribute counts
    if (n >= 4 && std::memcmp(d, "Bgeo", 4) != 0) {
        if (d[0] == 0x7f && d[1] == 'N' && d[2] == 'S' && d[3] == 'J')
            return fail(err, "new (JSON) BGEO format: only the classic version 5 format is read");
        return fail(err, "not a BGEO file (magic)");
    }
    if (n < 41) return 1;
    int32_t v[9];
    for (int k = 0; k < 9; ++k) v[k] = (int32_t)be32(d + 5 + 4 * k);
    if (v[0] != 5) return fail(err, "BGEO version must be 5");
    const int32_t points = v[1], nattr = v[5];
    if (points < 0 || nattr < 0) return fail(err, "negative point or attribute count");
    size_t at = 41;
    uint64_t words = 4;  // x y z w
    for (int32_t a = 0; a < nattr; ++a) {
        if (n - at < 2) return 1;
        const size_t name = be16(d + at);
        at += 2;
        if (n - at < name + 6) return 1;
        at += name;
        const uint32_t size = be16(d + at);
        const int32_t type = (int32_t)be32(d + at + 2);
        at += 6;
        if (type == 0 || type == 1 || type == 5) {  // float, int, vector: `size` default words
            if (n - at < 4ull * size) return 1;
            at += 4ull * size;
        } else if (type == 4) {  // indexed string: the string table
            if (n - at < 4) return 1;
            const int32_t nidx = (int32_t)be32(d + at);
            at += 4;
            if (nidx < 0) return fail(err, "negative string table size");
            for (int32_t k = 0; k < nidx; ++k) {
                if (n - at < 2) return 1;
                const size_t len = be16(d + at);
                at += 2;
                if (n - at < len) return 1;
                at += len;
            }
        } else if (type == 2) {
            return fail(err, "string point attributes (type 2) are not supported");
        } else {
            return fail(err, "unknown point attribute type " + std::to_string(type));
        }
        words += size;
    }
    if (words > (1u << 20)) return fail(err, "point records are too wide");
    L.points = (uint64_t)points;
    L.words = (uint32_t)words;
    L.attributes = (uint32_t)nattr;
    L.data_offset = at;
    if (need_points && (uint64_t)(n - at) / (4 * words) < L.points) return fail(err, "BGEO point data is truncated");
    return 0;
}

int bgeo_load(const char* path, bool header_only, BgeoFile& f, std::string& err) {
    f = BgeoFile();
    if (!header_only) {
        if (read_file(path, 0, f.raw, f.file_bytes, err)) return -1;
        f.compressed = is_gzip(f.raw.data(), f.raw.size());
        if (f.compressed) {
            if (gunzip(f.raw.data(), f.raw.size(), f.inflated, 0, err)) return -1;
            f.raw.clear();
            f.raw.shrink_to_fit();
            f.data = f.inflated.data();
            f.size = f.inflated.size();
        } else {
            f.data = f.raw.data();
            f.size = f.raw.size();
        }
        const int r = bgeo_layout(f.data, f.size, true, f.layout, err);
        if (r == 1) return fail(err, "BGEO header is truncated");
        return r;
    }
    // header only: a prefix of the file, grown until the header fits
    for (size_t chunk = 1 << 20;; chunk *= 8) {
        if (read_file(path, chunk, f.raw, f.file_bytes, err)) return -1;
        const bool whole = f.raw.size() == f.file_bytes;
        f.compressed = is_gzip(f.raw.data(), f.raw.size());
        int r;
        if (f.compressed) {
            std::string e2;
            const int g = gunzip(f.raw.data(), f.raw.size(), f.inflated, chunk / 4, e2);
            if (g != 0 && whole) return fail(err, e2);
            if (g != 0) continue;  // the prefix ran out before the header: read more
            f.data = f.inflated.data();
            f.size = f.inflated.size();
            r = bgeo_layout(f.data, f.size, false, f.layout, err);
            if (r == 1 && whole && f.size < chunk / 4) return fail(err, "BGEO header is truncated");
        } else {
            f.data = f.raw.data();
            f.size = f.raw.size();
            r = bgeo_layout(f.data, f.size, false, f.layout, err);
            if (r == 1 && whole) return fail(err, "BGEO header is truncated");
        }
        if (r == 0) return check_point_block(path, f, err);
        if (r < 0) return r;
    }
}

void bgeo_positions(const BgeoFile& f, float* xyz, uint64_t count) {
    const uint8_t* rec = f.data + f.layout.data_offset;
    const uint64_t stride = 4ull * f.layout.words;
    for (uint64_t i = 0; i < count; ++i)
        for (int c = 0; c < 3; ++c) {
            const uint32_t w = be32(rec + i * stride + 4 * c);
            std::memcpy(xyz + 3 * i + c, &w, 4);
        }
}

}  // namespace io

namespace {

// one thread per position word: byte-swap word c of record i into xyz[3i + c]
__global__ void k_bgeo_xyz(const uint32_t* __restrict__ rec, uint32_t words, uint64_t n, float* __restrict__ xyz) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * n) return;
    const uint64_t i = t / 3, c = t - 3 * i;
    xyz[t] = __uint_as_float(__byte_perm(rec[i * words + c], 0, 0x0123));
}

void fill_info(const io::BgeoFile& f, fm_bgeo_info* info) {
    if (!info) return;
    std::memset(info, 0, sizeof(*info));
    info->points = f.layout.points;
    info->record_words = f.layout.words;
    info->attributes = f.layout.attributes;
    info->file_bytes = f.file_bytes;
    info->data_bytes = f.compressed ? (uint64_t)f.inflated.size() : f.file_bytes;
    info->compressed = f.compressed ? 1 : 0;
}

void copy_err(const std::string& e, char* err, uint64_t err_len) {
    if (!err || err_len == 0) return;
    const size_t k = std::min<size_t>(e.size(), (size_t)err_len - 1);
    std::memcpy(err, e.data(), k);
    err[k] = 0;
}

// Decoded frame -> device positions -> scene (created, rebuilt in place, or
// replaced when it is too small or has another support radius).
int frame_to_scene(fm_ctx* ctx, const io::BgeoFile& f, float support, fm_scene** scene) {
    const uint64_t n = f.layout.points;
    if (n == 0) return set_err(ctx, FM_ERR_INVALID, "the particle file has no points");
    cudaSetDevice(ctx->device);
    const size_t rec_bytes = (size_t)n * f.layout.words * 4;
    if (!grow_buf(ctx->file_rec, rec_bytes) || !grow_buf(ctx->file_xyz, (size_t)n * 12))
        return set_err(ctx, FM_ERR_OOM, "particle-file buffer allocation failed");
    FM_CUDA(ctx, cudaMemcpyAsync(ctx->file_rec.p, f.data + f.layout.data_offset, rec_bytes, cudaMemcpyHostToDevice,
                                 ctx->stream));
    k_bgeo_xyz<<<(unsigned)((3 * n + 255) / 256), 256, 0, ctx->stream>>>((const uint32_t*)ctx->file_rec.p,
                                                                          f.layout.words, n, (float*)ctx->file_xyz.p);
    FM_CUDA(ctx, cudaGetLastError());
    const float* xyz = (const float*)ctx->file_xyz.p;
    fm_scene* s = *scene;
    if (s && s->ctx == ctx && s->capacity >= n && s->support == support)
        return fm_scene_update(s, xyz, n, 3, FM_MEM_DEVICE);
    fm_scene* fresh = nullptr;
    const int rc = fm_scene_create(ctx, xyz, n, 3, support, FM_MEM_DEVICE, &fresh);
    if (rc) return rc;
    if (s) fm_scene_destroy(s);
    *scene = fresh;
    return FM_OK;
}

}  // namespace
}  // namespace fm

// ---- numbered series --------------------------------------------------------

struct fm_dataset {
    std::vector<std::string> files;
    std::vector<int64_t> points;  // per frame, -1 until its header is read
    int window = 0;               // frames decoded ahead of the last one asked for
    std::mutex mu;
    std::condition_variable cv;
    struct Slot {
        int state = 0;  // 0 queued, 1 decoding, 2 ready, 3 failed
        std::shared_ptr<fm::io::BgeoFile> file;
        std::string err;
    };
    std::map<int, Slot> cache;
    std::deque<int> queue;
    std::vector<std::thread> workers;
    bool stop = false;
    std::string err;

    void work() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || !queue.empty(); });
            if (stop) return;
            const int i = queue.front();
            queue.pop_front();
            auto it = cache.find(i);
            if (it == cache.end() || it->second.state != 0) continue;  // evicted or taken meanwhile
            it->second.state = 1;
            lk.unlock();
            auto f = std::make_shared<fm::io::BgeoFile>();
            std::string e;
            const int rc = fm::io::bgeo_load(files[i].c_str(), false, *f, e);
            lk.lock();
            auto jt = cache.find(i);
            if (jt != cache.end()) {
                jt->second.state = rc ? 3 : 2;
                jt->second.file = rc ? nullptr : f;
                jt->second.err = e;
            }
            if (!rc) points[i] = (int64_t)f->layout.points;
            cv.notify_all();
        }
    }

    // decoded frame i (waits for a thread that is decoding it, or decodes it
    // here); then queues the next `window` frames and drops the others.  A slot
    // being decoded is never dropped; a finished one may be dropped by another
    // reader before a waiter wakes, and is then decoded again.
    std::shared_ptr<fm::io::BgeoFile> get(int i, std::string& e) {
        std::unique_lock<std::mutex> lk(mu);
        std::shared_ptr<fm::io::BgeoFile> f;
        for (;;) {
            auto it = cache.find(i);
            if (it != cache.end() && it->second.state >= 2) {
                f = it->second.file;
                e = it->second.err;
                break;
            }
            if (it != cache.end() && it->second.state == 1) {
                cv.wait(lk);
                continue;
            }
            cache[i].state = 1;  // absent or only queued: decode it here
            lk.unlock();
            auto nf = std::make_shared<fm::io::BgeoFile>();
            std::string le;
            const int rc = fm::io::bgeo_load(files[i].c_str(), false, *nf, le);
            lk.lock();
            Slot& sl = cache[i];
            sl.state = rc ? 3 : 2;
            sl.file = rc ? nullptr : nf;
            sl.err = le;
            if (!rc) points[i] = (int64_t)nf->layout.points;
            cv.notify_all();
            f = sl.file;
            e = le;
            break;
        }
        // keep [i, i + window]; queue what is missing of it
        for (auto jt = cache.begin(); jt != cache.end();) {
            const bool keep = jt->first >= i && jt->first <= i + window && jt->second.state != 3;
            if (!keep && jt->second.state != 1)
                jt = cache.erase(jt);
            else
                ++jt;
        }
        if (!workers.empty())
            for (int k = i + 1; k <= i + window && k < (int)files.size(); ++k)
                if (cache.find(k) == cache.end()) {
                    cache[k].state = 0;
                    queue.push_back(k);
                }
        cv.notify_all();
        return f;
    }

    int header(int i, fm_bgeo_info* info, std::string& e) {
        fm::io::BgeoFile f;
        if (fm::io::bgeo_load(files[i].c_str(), true, f, e)) return FM_ERR_INVALID;
        {
            std::lock_guard<std::mutex> lk(mu);
            points[i] = (int64_t)f.layout.points;
        }
        if (info) {
            fm::fill_info(f, info);
            info->data_bytes = 0;  // unknown without decoding the whole file
        }
        return FM_OK;
    }
};

extern "C" {

int fm_gunzip(const void* in, uint64_t in_len, void* out, uint64_t out_cap, uint64_t* out_len) {
    if (!in || !out_len || (!out && out_cap)) return FM_ERR_INVALID;
    try {
        std::vector<uint8_t> v;
        std::string e;
        if (fm::io::gunzip((const uint8_t*)in, (size_t)in_len, v, 0, e)) return FM_ERR_INVALID;
        *out_len = v.size();
        if (v.size() > out_cap) return FM_ERR_INVALID;
        if (!v.empty()) std::memcpy(out, v.data(), v.size());
        return FM_OK;
    } catch (const std::bad_alloc&) {
        return FM_ERR_OOM;
    }
}

int fm_bgeo_read(const char* path, float* xyz, uint64_t capacity, fm_bgeo_info* info, char* err, uint64_t err_len) {
    if (!path) {
        fm::copy_err("NULL path", err, err_len);
        return FM_ERR_INVALID;
    }
    try {
        fm::io::BgeoFile f;
        std::string e;
        if (fm::io::bgeo_load(path, xyz == nullptr, f, e)) {
            fm::copy_err(e, err, err_len);
            return FM_ERR_INVALID;
        }
        fm::fill_info(f, info);
        if (xyz) {
            fm::io::bgeo_positions(f, xyz, std::min<uint64_t>(capacity, f.layout.points));
        } else if (info) {
            info->data_bytes = 0;
        }
        return FM_OK;
    } catch (const std::bad_alloc&) {
        fm::copy_err("out of host memory", err, err_len);
        return FM_ERR_OOM;
    }
}

int fm_scene_create_bgeo(fm_ctx* ctx, const char* path, float support_radius, fm_scene** out) {
    if (!ctx) return FM_ERR_INVALID;
    if (!path || !out) return fm::set_err(ctx, FM_ERR_INVALID, "NULL argument");
    try {
        fm::io::BgeoFile f;
        std::string e;
        if (fm::io::bgeo_load(path, false, f, e)) return fm::set_err(ctx, FM_ERR_INVALID, e);
        *out = nullptr;
        const int rc = fm::frame_to_scene(ctx, f, support_radius, out);
        if (rc == FM_OK) FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host file buffer goes away
        return rc;
    } catch (const std::bad_alloc&) {
        return fm::set_err(ctx, FM_ERR_OOM, "out of host memory");
    }
}

int fm_dataset_open(const char* prefix, const char* suffix, int32_t count, int32_t threads, fm_dataset** out,
                    char* err, uint64_t err_len) {
    if (!prefix || !suffix || !out || threads < 0) {
        fm::copy_err("invalid argument", err, err_len);
        return FM_ERR_INVALID;
    }
    auto* ds = new (std::nothrow) fm_dataset();
    if (!ds) return FM_ERR_OOM;
    for (int64_t i = 1; count < 0 || i <= count; ++i) {
        std::string path = std::string(prefix) + std::to_string(i) + suffix;
        std::error_code ec;
        if (!std::filesystem::exists(path, ec)) break;
        ds->files.push_back(path);
    }
    ds->points.assign(ds->files.size(), -1);
    ds->window = threads > 0 ? 2 * threads : 0;
    for (int t = 0; t < threads; ++t) ds->workers.emplace_back([ds] { ds->work(); });
    *out = ds;
    return FM_OK;
}

int32_t fm_dataset_frames(const fm_dataset* ds) { return ds ? (int32_t)ds->files.size() : 0; }

const char* fm_dataset_path(const fm_dataset* ds, int32_t i) {
    if (!ds || i < 0 || i >= (int32_t)ds->files.size()) return nullptr;
    return ds->files[i].c_str();
}

const char* fm_dataset_last_error(const fm_dataset* ds) { return ds ? ds->err.c_str() : "no dataset"; }

int fm_dataset_frame_info(fm_dataset* ds, int32_t i, fm_bgeo_info* info) {
    if (!ds) return FM_ERR_INVALID;
    if (i < 0 || i >= (int32_t)ds->files.size()) {
        ds->err = "frame index out of range";
        return FM_ERR_INVALID;
    }
    try {
        return ds->header(i, info, ds->err);
    } catch (const std::bad_alloc&) {
        ds->err = "out of host memory";
        return FM_ERR_OOM;
    }
}

int fm_dataset_max_particles(fm_dataset* ds, uint64_t* out) {
    if (!ds || !out) return FM_ERR_INVALID;
    uint64_t m = 0;
    for (int32_t i = 0; i < (int32_t)ds->files.size(); ++i) {
        int64_t p;
        {
            std::lock_guard<std::mutex> lk(ds->mu);
            p = ds->points[i];
        }
        if (p < 0) {
            const int rc = fm_dataset_frame_info(ds, i, nullptr);
            if (rc) return rc;
            std::lock_guard<std::mutex> lk(ds->mu);
            p = ds->points[i];
        }
        m = std::max<uint64_t>(m, (uint64_t)p);
    }
    *out = m;
    return FM_OK;
}

int fm_dataset_read(fm_dataset* ds, int32_t i, float* xyz, uint64_t capacity, uint64_t* n) {
    if (!ds) return FM_ERR_INVALID;
    if (i < 0 || i >= (int32_t)ds->files.size()) {
        ds->err = "frame index out of range";
        return FM_ERR_INVALID;
    }
    try {
        std::string e;
        auto f = ds->get(i, e);
        if (!f) {
            ds->err = e;
            return FM_ERR_INVALID;
        }
        if (n) *n = f->layout.points;
        if (xyz) fm::io::bgeo_positions(*f, xyz, std::min<uint64_t>(capacity, f->layout.points));
        return FM_OK;
    } catch (const std::bad_alloc&) {
        ds->err = "out of host memory";
        return FM_ERR_OOM;
    }
}

int fm_dataset_scene(fm_dataset* ds, fm_ctx* ctx, int32_t i, float support_radius, fm_scene** scene) {
    if (!ctx) return FM_ERR_INVALID;
    if (!ds || !scene) return fm::set_err(ctx, FM_ERR_INVALID, "NULL argument");
    if (i < 0 || i >= (int32_t)ds->files.size()) return fm::set_err(ctx, FM_ERR_INVALID, "frame index out of range");
    try {
        std::string e;
        auto f = ds->get(i, e);
        if (!f) return fm::set_err(ctx, FM_ERR_INVALID, e);
        const int rc = fm::frame_to_scene(ctx, *f, support_radius, scene);
        if (rc == FM_OK) FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // f may be dropped from the cache
        return rc;
    } catch (const std::bad_alloc&) {
        return fm::set_err(ctx, FM_ERR_OOM, "out of host memory");
    }
}

void fm_dataset_close(fm_dataset* ds) {
    if (!ds) return;
    {
        std::lock_guard<std::mutex> lk(ds->mu);
        ds->stop = true;
    }
    ds->cv.notify_all();
    for (auto& t : ds->workers) t.join();
    delete ds;
}

}  // extern "C"
