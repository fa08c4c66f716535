// State files: the particle records of a simulation plus what resuming it needs, for reproducible
// initial states, golden vectors and restarts.  The reference keeps its whole simulation state in
// the particle buffer (Particle.h:8-31; PBFSolver::step re-reads it every frame), so the records
// plus the solver parameters determine every later step; the optional sections carry what this
// library keeps beside them (the per-particle lambda sums of the warm start, and the scenes of a
// batch).
//
// Layout (little-endian, as in memory on the supported hosts):
//   header           256 bytes (akua_state_header, zero-padded)
//   records          numParticles * 108 bytes, akua_particle
//   lambda sums      numParticles * 4 bytes       if sections & AKUA_STATE_LAMBDA_SUMS
//   scenes           numScenes * 40 bytes         if numScenes > 0 (akua_scene_desc)
// `crc32` is the CRC-32 (IEEE 802.3 polynomial, reflected, as in zlib) of everything after the
// header.
#include <cstdio>
#include <cstring>
#include <vector>

#include "akua_pbf.h"

static_assert(sizeof(akua_state_header) == AKUA_STATE_HEADER_BYTES, "state header size");
static_assert(sizeof(akua_particle) == 108, "record size");
static_assert(sizeof(akua_scene_desc) == 40, "scene descriptor size");

namespace {

struct Crc32 {
    uint32_t table[256];
    Crc32() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
    }
    uint32_t update(uint32_t crc, const void* data, size_t bytes) const {
        const unsigned char* p = static_cast<const unsigned char*>(data);
        crc = ~crc;
        for (size_t i = 0; i < bytes; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
        return ~crc;
    }
};

const Crc32& crc() {
    static const Crc32 c;
    return c;
}

const char kMagic[8] = {'A', 'K', 'U', 'A', 'P', 'B', 'F', '\0'};

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

int check_header(const akua_state_header& h) {
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != AKUA_STATE_VERSION ||
        h.recordBytes != sizeof(akua_particle) || h.numParticles <= 0 || h.numScenes < 0)
        return AKUA_ERR_INVALID_ARGUMENT;
    return AKUA_OK;
}

}  // namespace

extern "C" {

void akua_state_init_header(akua_state_header* h) {
    if (!h) return;
    std::memset(h, 0, sizeof(*h));
    std::memcpy(h->magic, kMagic, 8);
    h->version = AKUA_STATE_VERSION;
    h->recordBytes = sizeof(akua_particle);
}

int akua_state_save(const char* path, const akua_state_header* header, const void* records,
                    const float* lambdaSums, const akua_scene_desc* scenes) {
    if (!path || !header || !records) return AKUA_ERR_INVALID_ARGUMENT;
    akua_state_header h = *header;
    if (check_header(h) != AKUA_OK) return AKUA_ERR_INVALID_ARGUMENT;
    if ((lambdaSums != nullptr) != ((h.sections & AKUA_STATE_LAMBDA_SUMS) != 0))
        return AKUA_ERR_INVALID_ARGUMENT;
    if ((scenes != nullptr) != (h.numScenes > 0)) return AKUA_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)h.numParticles;
    uint32_t c = crc().update(0u, records, n * sizeof(akua_particle));
    if (lambdaSums) c = crc().update(c, lambdaSums, n * sizeof(float));
    if (scenes) c = crc().update(c, scenes, (size_t)h.numScenes * sizeof(akua_scene_desc));
    h.crc32 = c;
    File f;
    f.f = std::fopen(path, "wb");
    if (!f.f) return AKUA_ERR_INVALID_ARGUMENT;
    bool ok = std::fwrite(&h, sizeof(h), 1, f.f) == 1 &&
              std::fwrite(records, sizeof(akua_particle), n, f.f) == n;
    if (ok && lambdaSums) ok = std::fwrite(lambdaSums, sizeof(float), n, f.f) == n;
    if (ok && scenes)
        ok = std::fwrite(scenes, sizeof(akua_scene_desc), (size_t)h.numScenes, f.f) ==
             (size_t)h.numScenes;
    ok = ok && std::fflush(f.f) == 0;
    return ok ? AKUA_OK : AKUA_ERR_INVALID_ARGUMENT;
}

int akua_state_read_header(const char* path, akua_state_header* header) {
    if (!path || !header) return AKUA_ERR_INVALID_ARGUMENT;
    File f;
    f.f = std::fopen(path, "rb");
    if (!f.f) return AKUA_ERR_INVALID_ARGUMENT;
    if (std::fread(header, sizeof(*header), 1, f.f) != 1) return AKUA_ERR_INVALID_ARGUMENT;
    return check_header(*header);
}

int akua_state_load(const char* path, akua_state_header* header, void* records,
                    int64_t capacity, float* lambdaSums, akua_scene_desc* scenes,
                    int32_t sceneCapacity) {
    if (!path || !header || !records) return AKUA_ERR_INVALID_ARGUMENT;
    File f;
    f.f = std::fopen(path, "rb");
    if (!f.f) return AKUA_ERR_INVALID_ARGUMENT;
    akua_state_header h;
    if (std::fread(&h, sizeof(h), 1, f.f) != 1 || check_header(h) != AKUA_OK)
        return AKUA_ERR_INVALID_ARGUMENT;
    if (h.numParticles > capacity) return AKUA_ERR_TOO_LARGE;
    if (h.numScenes > 0 && (!scenes || h.numScenes > sceneCapacity)) return AKUA_ERR_TOO_LARGE;
    const size_t n = (size_t)h.numParticles;
    if (std::fread(records, sizeof(akua_particle), n, f.f) != n) return AKUA_ERR_INVALID_ARGUMENT;
    uint32_t c = crc().update(0u, records, n * sizeof(akua_particle));
    std::vector<float> sums;
    if (h.sections & AKUA_STATE_LAMBDA_SUMS) {
        sums.resize(n);
        if (std::fread(sums.data(), sizeof(float), n, f.f) != n) return AKUA_ERR_INVALID_ARGUMENT;
        c = crc().update(c, sums.data(), n * sizeof(float));
        if (lambdaSums) std::memcpy(lambdaSums, sums.data(), n * sizeof(float));
    }
    if (h.numScenes > 0) {
        const size_t k = (size_t)h.numScenes;
        if (std::fread(scenes, sizeof(akua_scene_desc), k, f.f) != k)
            return AKUA_ERR_INVALID_ARGUMENT;
        c = crc().update(c, scenes, k * sizeof(akua_scene_desc));
    }
    if (c != h.crc32) return AKUA_ERR_CORRUPT;
    *header = h;
    return AKUA_OK;
}

}  // extern "C"
