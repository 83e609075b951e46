// persist.cu -- map dump in the reference's raw layout (host code only).
//
// MapStruct<false>::writeToDisk / readFromDisk (src/data_struct/map_struct.cu:535-613)
// dump the host mirror of the reference's map storage as one binary file plus
// "<name>.txt" holding the MapSize.  The file is the memory image of the
// reference's chained hash map; this library keeps an open-addressing table,
// so the writer rebuilds the chained form and the reader scans it back into
// per-block arrays, which then go through gbf_map_export / gbf_map_import.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "gbf_internal.h"

namespace gbf {
namespace {

// include/data_struct/voxel.h:20-22: short sdf; float weight; uchar3 rgb (natural alignment: 12 B)
struct RefVoxel {
    int16_t sdf;
    int16_t pad0;
    float weight;
    uint8_t rgb[3];
    uint8_t pad1;
};
// include/data_struct/hash_entry.h:20-22: int ptr_; int offset_; Vector3i pos_ (20 B)
struct RefEntry {
    int32_t ptr, offset, pos[3];
};
static_assert(sizeof(RefVoxel) == 12, "reference Voxel is 12 bytes");
static_assert(sizeof(RefEntry) == 20, "reference HashEntry is 20 bytes");

constexpr int kVox = 512;  // BLOCK_SIZE3 (include/data_struct/map_struct.h:9)

// MapStruct() defaults (src/data_struct/map_struct.cu:19-21)
constexpr gbf_map_size kDefaultSize = {200000, 250000, 200000};

// computeHash (src/data_struct/map_struct.cu:143-148): int32 products with
// wraparound, C remainder, made non-negative.  Unsigned arithmetic gives the
// same bits without signed overflow.
int ref_hash(int x, int y, int z, int n) {
    const int h = (int)(((unsigned)x * 73856093u) ^ ((unsigned)y * 19349669u) ^ ((unsigned)z * 83492791u));
    const int r = h % n;
    return r < 0 ? r + n : r;
}

// Voxel::setSDF = packFloat = (short)(val * 32767) (voxel.h:41-44); values outside [-1, 1]
// (which the integration never stores) are clamped instead of overflowing.
int16_t pack_sdf(float v) {
    float t = v * 32767.f;
    if (!(t > -32768.f)) t = -32768.f;
    if (t > 32767.f) t = 32767.f;
    return (int16_t)t;
}

bool size_ok(const gbf_map_size &z) {
    return z.num_blocks > 0 && z.num_buckets > 0 && z.num_hash_entries >= z.num_buckets &&
           (long long)z.num_blocks * kVox <= 0x7fffffffLL;  // MapState::num_total_voxels is an int
}

long long dump_bytes(const gbf_map_size &z) {
    return (long long)z.num_blocks * kVox * (long long)sizeof(RefVoxel) +
           (long long)z.num_hash_entries * (long long)sizeof(RefEntry) + 4LL * z.num_blocks + 4LL * z.num_buckets + 8;
}

struct File {
    FILE *f = nullptr;
    explicit File(FILE *p) : f(p) {}
    ~File() {
        if (f) fclose(f);
    }
};

bool seek(FILE *f, long long off) {
    return fseeko(f, (off_t)off, SEEK_SET) == 0;
}

}  // namespace
}  // namespace gbf

using namespace gbf;

extern "C" {

GBF_API gbf_status gbf_dump_write(const char *path, const gbf_map_size *size, const int32_t *coords,
                                  const float *sdf, const float *weight, const uint8_t *rgb, int64_t n_blocks) {
    if (!path || n_blocks < 0 || (n_blocks > 0 && (!coords || !sdf || !weight || !rgb)))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_dump_write: null or negative argument");
    const gbf_map_size z = size ? *size : kDefaultSize;
    if (!size_ok(z)) return set_error(GBF_ERR_INVALID_ARG, "gbf_dump_write: invalid map size");
    if (n_blocks > z.num_blocks) return set_error(GBF_ERR_CAPACITY, "gbf_dump_write: more blocks than num_blocks");

    // chained table: home buckets [0, num_buckets), excess entries after them
    std::vector<RefEntry> table((size_t)z.num_hash_entries, RefEntry{-1, -1, {0, 0, 0}});
    const int excess = z.num_hash_entries - z.num_buckets;
    int next_offset = 1;
    for (int64_t b = 0; b < n_blocks; ++b) {
        const int x = coords[3 * b], y = coords[3 * b + 1], zc = coords[3 * b + 2];
        int cur = ref_hash(x, y, zc, z.num_buckets);
        for (int i = cur;;) {  // findEntry (map_struct.cu:365-380): a block may appear once
            const RefEntry &e = table[i];
            if (e.ptr != -1 && e.pos[0] == x && e.pos[1] == y && e.pos[2] == zc)
                return set_error(GBF_ERR_INVALID_ARG, "gbf_dump_write: duplicate block position");
            if (e.offset <= 0) break;
            i = z.num_buckets + e.offset - 1;
        }
        const RefEntry fresh{(int32_t)(b * kVox), -1, {x, y, zc}};
        if (table[cur].ptr == -1) {
            table[cur] = fresh;
            continue;
        }
        while (table[cur].offset > 0) cur = z.num_buckets + table[cur].offset - 1;
        if (next_offset > excess) return set_error(GBF_ERR_CAPACITY, "gbf_dump_write: excess entries exhausted");
        RefEntry &slot = table[(size_t)z.num_buckets + next_offset - 1];
        slot = fresh;
        slot.offset = 0;  // createBlock gives a new excess entry offset 0 (map_struct.cu:319)
        table[cur].offset = next_offset++;
    }

    File out(fopen(path, "wb"));
    if (!out.f) return set_error(GBF_ERR_IO, "gbf_dump_write: cannot open file");
    bool ok = true;
    // voxels: written blocks first, the rest of the pool zero (MapStruct::reset memsets it)
    const int chunk = 256;
    std::vector<RefVoxel> buf((size_t)chunk * kVox);
    for (long long first = 0; ok && first < z.num_blocks; first += chunk) {
        const int cnt = (int)std::min<long long>(chunk, z.num_blocks - first);
        std::memset(buf.data(), 0, buf.size() * sizeof(RefVoxel));
        for (int k = 0; k < cnt; ++k) {
            const long long b = first + k;
            if (b >= n_blocks) break;
            for (int i = 0; i < kVox; ++i) {
                const size_t src = (size_t)b * kVox + i;
                RefVoxel &v = buf[(size_t)k * kVox + i];
                v.sdf = pack_sdf(sdf[src]);
                v.weight = weight[src];
                v.rgb[0] = rgb[3 * src];
                v.rgb[1] = rgb[3 * src + 1];
                v.rgb[2] = rgb[3 * src + 2];
            }
        }
        ok = fwrite(buf.data(), sizeof(RefVoxel), (size_t)cnt * kVox, out.f) == (size_t)cnt * kVox;
    }
    if (ok) ok = fwrite(table.data(), sizeof(RefEntry), table.size(), out.f) == table.size();
    // heap after n pops from the initial stack heap[i] = N - i - 1 (map_struct.cu:58-69)
    std::vector<int32_t> heap((size_t)z.num_blocks);
    for (int i = 0; i < z.num_blocks; ++i) heap[i] = z.num_blocks - i - 1;
    if (ok) ok = fwrite(heap.data(), 4, heap.size(), out.f) == heap.size();
    std::vector<int32_t> mutex((size_t)z.num_buckets, 0);
    if (ok) ok = fwrite(mutex.data(), 4, mutex.size(), out.f) == mutex.size();
    const int32_t counters[2] = {(int32_t)(z.num_blocks - 1 - n_blocks), next_offset};
    if (ok) ok = fwrite(counters, 4, 2, out.f) == 2;
    if (ok) ok = fflush(out.f) == 0;
    if (!ok) return set_error(GBF_ERR_IO, "gbf_dump_write: write failed");

    File txt(fopen((std::string(path) + ".txt").c_str(), "wb"));
    if (!txt.f) return set_error(GBF_ERR_IO, "gbf_dump_write: cannot open the .txt file");
    const int32_t ms[3] = {z.num_blocks, z.num_hash_entries, z.num_buckets};  // MapSize field order
    if (fwrite(ms, 4, 3, txt.f) != 3 || fflush(txt.f) != 0)
        return set_error(GBF_ERR_IO, "gbf_dump_write: .txt write failed");
    return GBF_OK;
}

GBF_API gbf_status gbf_dump_read(const char *path, gbf_map_size *size, int32_t *coords, float *sdf, float *weight,
                                 uint8_t *rgb, int64_t max_blocks, int64_t *n_blocks) {
    if (!path || !n_blocks || (coords && (!sdf || !weight || !rgb || max_blocks < 0)))
        return set_error(GBF_ERR_INVALID_ARG, "gbf_dump_read: null argument");
    gbf_map_size z = kDefaultSize;  // the reference reads with its defaults when the .txt is absent
    {
        File txt(fopen((std::string(path) + ".txt").c_str(), "rb"));
        if (txt.f) {
            int32_t ms[3];
            if (fread(ms, 4, 3, txt.f) != 3) return set_error(GBF_ERR_IO, "gbf_dump_read: short .txt file");
            z = gbf_map_size{ms[0], ms[1], ms[2]};
        }
    }
    if (!size_ok(z)) return set_error(GBF_ERR_IO, "gbf_dump_read: invalid map size in the .txt file");
    File in(fopen(path, "rb"));
    if (!in.f) return set_error(GBF_ERR_IO, "gbf_dump_read: cannot open file");
    if (fseeko(in.f, 0, SEEK_END) != 0) return set_error(GBF_ERR_IO, "gbf_dump_read: seek failed");
    if ((long long)ftello(in.f) != dump_bytes(z))
        return set_error(GBF_ERR_IO, "gbf_dump_read: file size does not match the map size");

    const long long entries_at = (long long)z.num_blocks * kVox * (long long)sizeof(RefVoxel);
    std::vector<RefEntry> table((size_t)z.num_hash_entries);
    if (!seek(in.f, entries_at) || fread(table.data(), sizeof(RefEntry), table.size(), in.f) != table.size())
        return set_error(GBF_ERR_IO, "gbf_dump_read: short file");

    std::vector<const RefEntry *> blocks;
    std::set<std::tuple<int, int, int>> seen;
    for (const RefEntry &e : table) {
        if (e.ptr == -1) continue;
        if (e.ptr < 0 || e.ptr % kVox || e.ptr / kVox >= z.num_blocks)
            return set_error(GBF_ERR_IO, "gbf_dump_read: hash entry points outside the block pool");
        if (seen.insert(std::make_tuple(e.pos[0], e.pos[1], e.pos[2])).second) blocks.push_back(&e);
    }
    if (size) *size = z;
    *n_blocks = (int64_t)blocks.size();
    if (!coords) return GBF_OK;

    std::vector<RefVoxel> buf(kVox);
    const int64_t n = std::min<int64_t>(max_blocks, (int64_t)blocks.size());
    for (int64_t b = 0; b < n; ++b) {
        const RefEntry &e = *blocks[b];
        coords[3 * b] = e.pos[0];
        coords[3 * b + 1] = e.pos[1];
        coords[3 * b + 2] = e.pos[2];
        if (!seek(in.f, (long long)e.ptr * (long long)sizeof(RefVoxel)) ||
            fread(buf.data(), sizeof(RefVoxel), kVox, in.f) != (size_t)kVox)
            return set_error(GBF_ERR_IO, "gbf_dump_read: short file");
        for (int i = 0; i < kVox; ++i) {
            const size_t o = (size_t)b * kVox + i;
            sdf[o] = buf[i].sdf / (float)32767;  // Voxel::getSDF / unpackFloat (voxel.h:36-39)
            weight[o] = buf[i].weight;
            rgb[3 * o] = buf[i].rgb[0];
            rgb[3 * o + 1] = buf[i].rgb[1];
            rgb[3 * o + 2] = buf[i].rgb[2];
        }
    }
    return GBF_OK;
}

GBF_API gbf_status gbf_map_write_dump(gbf_session *s, const char *path, const gbf_map_size *size) {
    if (!s || !path) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_write_dump: null");
    int64_t n = 0;
    gbf_status st = gbf_map_export(s, nullptr, nullptr, nullptr, nullptr, 0, &n);
    if (st != GBF_OK) return st;
    std::vector<int32_t> c((size_t)n * 3);
    std::vector<float> sd((size_t)n * kVox), w((size_t)n * kVox);
    std::vector<uint8_t> rgb((size_t)n * kVox * 3);
    if (n > 0) {
        st = gbf_map_export(s, c.data(), sd.data(), w.data(), rgb.data(), n, &n);
        if (st != GBF_OK) return st;
    }
    return gbf_dump_write(path, size, c.data(), sd.data(), w.data(), rgb.data(), n);
}

GBF_API gbf_status gbf_map_read_dump(gbf_session *s, const char *path) {
    if (!s || !path) return set_error(GBF_ERR_INVALID_ARG, "gbf_map_read_dump: null");
    int64_t n = 0;
    gbf_status st = gbf_dump_read(path, nullptr, nullptr, nullptr, nullptr, nullptr, 0, &n);
    if (st != GBF_OK) return st;
    if (n > s->cfg.num_blocks) return set_error(GBF_ERR_CAPACITY, "gbf_map_read_dump: more blocks than the pool");
    std::vector<int32_t> c((size_t)n * 3);
    std::vector<float> sd((size_t)n * kVox), w((size_t)n * kVox);
    std::vector<uint8_t> rgb((size_t)n * kVox * 3);
    st = gbf_dump_read(path, nullptr, c.data(), sd.data(), w.data(), rgb.data(), n, &n);
    if (st != GBF_OK) return st;
    st = reset_map(s);
    if (st != GBF_OK) return st;
    return gbf_map_import(s, c.data(), sd.data(), w.data(), rgb.data(), n);
}

}  // extern "C"
