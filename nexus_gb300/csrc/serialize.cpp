// SEAL's byte format for a CKKS ciphertext (compr_mode_type::none), so the
// engine's ciphertexts can cross the client/server boundary NEXUS measures
// (src/matrix_mul.cpp:192-198 saves and loads SEAL ciphertexts).
//
// Layout (native/src/seal/serialization.h:60-93, ciphertext.cpp:190-248,
// dynarray.h:652-680): a 16-byte SEALHeader {magic 0xA15E, header size 16,
// version 4.1, compr_mode 0, reserved 0, total size}; parms_id (4 x uint64);
// is_ntt_form (1 byte); size, poly_modulus_degree, coeff_modulus_size
// (uint64 each); scale (double); correction_factor (uint64); then the
// coefficient array as its own serialized object: a second SEALHeader, the
// element count (uint64) and the words [size][coeff_modulus_size][N].
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../../include/nexus_gb300.h"
#include "context.h"

namespace {

constexpr uint16_t kMagic = 0xA15E;
constexpr uint8_t kHeaderSize = 16;
constexpr uint8_t kVersionMajor = 4;
constexpr uint8_t kVersionMinor = 1;

size_t saved_size(size_t words) { return 2 * kHeaderSize + 32 + 1 + 5 * 8 + 8 + words * 8; }

template <class T>
void put(uint8_t *&p, T v)
{
    std::memcpy(p, &v, sizeof(T));
    p += sizeof(T);
}

template <class T>
T get(const uint8_t *&p, const uint8_t *end)
{
    if ((size_t)(end - p) < sizeof(T)) throw std::invalid_argument("buffer is too small");
    T v;
    std::memcpy(&v, p, sizeof(T));
    p += sizeof(T);
    return v;
}

void put_header(uint8_t *&p, uint64_t size)
{
    put<uint16_t>(p, kMagic);
    put<uint8_t>(p, kHeaderSize);
    put<uint8_t>(p, kVersionMajor);
    put<uint8_t>(p, kVersionMinor);
    put<uint8_t>(p, 0);  // compr_mode_type::none
    put<uint16_t>(p, 0);
    put<uint64_t>(p, size);
}

// Serialization::Load's header checks (serialization.cpp): magic, header
// size, a 4.x version, no compression, and the declared size
uint64_t get_header(const uint8_t *&p, const uint8_t *end)
{
    if (get<uint16_t>(p, end) != kMagic) throw std::invalid_argument("loaded SEALHeader is invalid");
    if (get<uint8_t>(p, end) != kHeaderSize) throw std::invalid_argument("loaded SEALHeader is invalid");
    const uint8_t major = get<uint8_t>(p, end);
    get<uint8_t>(p, end);
    if (major != kVersionMajor) throw std::logic_error("incompatible version");
    if (get<uint8_t>(p, end) != 0) throw std::invalid_argument("unsupported compression mode");
    get<uint16_t>(p, end);
    return get<uint64_t>(p, end);
}

}  // namespace

extern "C" int nexus_seal_ciphertext_save(const uint64_t *words, int size, int limbs, int log_n, double scale,
                                          const uint64_t *parms_id, int is_ntt_form, uint8_t *out, size_t capacity,
                                          size_t *written)
{
    static const char *fn = "nexus_seal_ciphertext_save";
    if (!written || !parms_id) {
        nexus::set_error(std::string(fn) + ": null argument");
        return -1;
    }
    if (size < 2 || limbs < 1 || log_n < 1 || log_n > 17) {
        nexus::set_error(std::string(fn) + ": bad size, limbs or log_n");
        return -1;
    }
    const size_t n = size_t(1) << log_n;
    const size_t count = (size_t)size * limbs * n;
    const size_t total = saved_size(count);
    *written = total;
    if (!out) return 0;
    if (!words || capacity < total) {
        nexus::set_error(std::string(fn) + ": output buffer is too small");
        return -1;
    }
    uint8_t *p = out;
    put_header(p, total);
    for (int i = 0; i < 4; ++i) put<uint64_t>(p, parms_id[i]);
    put<uint8_t>(p, is_ntt_form ? 1 : 0);
    put<uint64_t>(p, (uint64_t)size);
    put<uint64_t>(p, (uint64_t)n);
    put<uint64_t>(p, (uint64_t)limbs);
    put<double>(p, scale);
    put<uint64_t>(p, 1);  // correction_factor (BGV only; 1 for CKKS)
    put_header(p, (uint64_t)(kHeaderSize + 8 + count * 8));
    put<uint64_t>(p, (uint64_t)count);
    std::memcpy(p, words, count * 8);
    return 0;
}

extern "C" int nexus_seal_ciphertext_load(const uint8_t *bytes, size_t len, uint64_t *words, size_t capacity_words,
                                          int *size, int *limbs, int *log_n, double *scale, uint64_t *parms_id,
                                          int *is_ntt_form)
{
    static const char *fn = "nexus_seal_ciphertext_load";
    if (!bytes || !size || !limbs || !log_n || !scale || !parms_id || !is_ntt_form) {
        nexus::set_error(std::string(fn) + ": null argument");
        return -1;
    }
    try {
        const uint8_t *p = bytes, *end = bytes + len;
        if (get_header(p, end) != len) throw std::invalid_argument("size indicated by loaded SEALHeader is out of bounds");
        for (int i = 0; i < 4; ++i) parms_id[i] = get<uint64_t>(p, end);
        const uint8_t ntt = get<uint8_t>(p, end);
        const uint64_t sz = get<uint64_t>(p, end), n = get<uint64_t>(p, end), l = get<uint64_t>(p, end);
        const double sc = get<double>(p, end);
        get<uint64_t>(p, end);  // correction_factor
        if (sz < 2 || sz > 16 || l < 1 || l > 64 || n < 2 || (n & (n - 1)) || n > (1u << 17))
            throw std::invalid_argument("ciphertext data is invalid");
        const uint64_t count = sz * l * n;
        const uint64_t inner = get_header(p, end);
        if (inner != kHeaderSize + 8 + count * 8) throw std::invalid_argument("ciphertext data is invalid");
        if (get<uint64_t>(p, end) != count) throw std::invalid_argument("ciphertext data is invalid");
        if ((size_t)(end - p) != count * 8) throw std::invalid_argument("buffer size does not match the header");
        int lg = 0;
        while ((uint64_t(1) << lg) < n) ++lg;
        *size = (int)sz;
        *limbs = (int)l;
        *log_n = lg;
        *scale = sc;
        *is_ntt_form = ntt ? 1 : 0;
        if (!words) return 0;
        if (capacity_words < count) throw std::invalid_argument("output buffer is too small");
        std::memcpy(words, p, count * 8);
    } catch (const std::exception &e) {
        nexus::set_error(std::string(fn) + ": " + e.what());
        return -1;
    }
    return 0;
}
