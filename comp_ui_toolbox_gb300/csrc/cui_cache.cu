// On-disk cache of the device-built tables, keyed by a hash of the setup
// (+auxiliary/compute_or_load_hash.m:65-185).
//
// The reference wraps each expensive table computation in compute_or_load_hash:
// the arguments are hashed into a file name (:57-73); an existing file whose
// stored arguments differ from the call's is a hash collision and an error
// (:90-107); a file holding the outputs is loaded (:112-131), otherwise the
// function runs and its outputs are saved beside the arguments (:133-185).
//
// Here the cached outputs are the two arrays cui_born_plan_create_setup computes
// on the device -- the lateral transfer-function table and the incident fields,
// both FP32 in the plan's device layout -- and the key is a canonical byte
// string of exactly the setup fields they depend on (grid, array, faces,
// medium, anti-aliasing, frequencies, per-wave frequency maps and normal
// velocities; not the receive mixes, which only shape host-side metadata, and
// not the device).  File: magic, key length, key, then each array's byte count
// and bytes.  It is written to a temporary name and renamed into place, so a
// reader never sees a partial file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cui_internal.cuh"

namespace cui {
namespace {

constexpr char kMagic[8] = {'C', 'U', 'I', 'T', 'B', 'L', '0', '1'};
constexpr size_t kChunk = size_t(64) << 20;  // bytes per staged host <-> device copy

template <typename T>
void put(std::vector<unsigned char>& k, const T& v) {
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&v);
    k.insert(k.end(), b, b + sizeof(T));
}

template <typename T>
void put_array(std::vector<unsigned char>& k, const T* v, size_t n) {
    put(k, static_cast<uint64_t>(n));
    const unsigned char* b = reinterpret_cast<const unsigned char*>(v);
    k.insert(k.end(), b, b + sizeof(T) * n);
}

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

// pinned staging buffer for the chunked copies (freed on scope exit)
struct Staging {
    void* h = nullptr;
    ~Staging() {
        if (h) cudaFreeHost(h);
    }
};

}  // namespace

cui_status setup_key(const cui_born_setup_desc* d, std::vector<unsigned char>& key) {
    if (!d) return set_error(CUI_ERR_INVALID_ARG, "desc is NULL");
    if (d->n_dims != 2 && d->n_dims != 3) return set_error(CUI_ERR_INVALID_ARG, "n_dims must be 2 or 3");
    if (d->n_f_unique < 1 || !d->f_unique) return set_error(CUI_ERR_INVALID_ARG, "f_unique is NULL or empty");
    if (d->n_measurements < 1 || !d->waves) return set_error(CUI_ERR_INVALID_ARG, "waves is NULL or empty");
    const int64_t E = static_cast<int64_t>(d->n_elements_axis[0]) * (d->n_dims == 3 ? d->n_elements_axis[1] : 1);
    if (E < 1) return set_error(CUI_ERR_INVALID_ARG, "no elements");
    key.clear();
    key.insert(key.end(), kMagic, kMagic + 8);
    put(key, d->n_dims);
    for (int a = 0; a < 3; ++a) put(key, d->n_points_axis[a]);
    for (int a = 0; a < 3; ++a) put(key, d->delta_axis[a]);
    put(key, d->z_start);
    for (int a = 0; a < 2; ++a) {
        put(key, d->n_elements_axis[a]);
        put(key, d->pitch_axis[a]);
        put(key, d->width_axis[a]);
        put(key, d->n_face_axis[a]);
    }
    const cui_absorption_desc& ab = d->absorption;  // field by field: no padding bytes in the key
    put(key, ab.kind);
    put(key, ab.c);
    put(key, ab.constant_db);
    put(key, ab.slope_db);
    put(key, ab.exponent);
    put(key, ab.f_ref);
    put(key, ab.dispersion);
    put(key, d->aa_tx_beta);
    put(key, d->aa_rx_beta);
    // face weights enter the key only when they are not uniform (keys of uniform setups unchanged)
    const bool focused = (d->lens_focus_axis[0] > 0.0 && std::isfinite(d->lens_focus_axis[0])) ||
                         (d->n_dims == 3 && d->lens_focus_axis[1] > 0.0 && std::isfinite(d->lens_focus_axis[1]));
    if (d->face_apodization || focused) {
        const char tag[8] = {'F', 'A', 'C', 'E', 'W', 'G', 'T', 'S'};
        key.insert(key.end(), tag, tag + 8);
        const size_t Q = static_cast<size_t>(std::max(1, d->n_face_axis[0])) *
                         (d->n_dims == 3 ? static_cast<size_t>(std::max(1, d->n_face_axis[1])) : 1);
        put(key, static_cast<int32_t>(d->face_apodization != nullptr));
        if (d->face_apodization) put_array(key, d->face_apodization, Q);
        put(key, d->lens_focus_axis[0]);
        put(key, d->lens_focus_axis[1]);
        put(key, d->lens_c);
    }
    put_array(key, d->f_unique, static_cast<size_t>(d->n_f_unique));
    put(key, d->n_measurements);
    for (int w = 0; w < d->n_measurements; ++w) {
        const cui_wave_desc& wd = d->waves[w];
        if (wd.n_f < 0 || (wd.n_f > 0 && (!wd.indices_f_to_unique || !wd.v_d)))
            return set_error(CUI_ERR_INVALID_ARG, "wave " + std::to_string(w) + " lacks its frequency map or v_d");
        put_array(key, wd.indices_f_to_unique, static_cast<size_t>(wd.n_f));
        for (int64_t i = 0; i < static_cast<int64_t>(wd.n_f) * E; ++i) {
            put(key, wd.v_d[i].re);
            put(key, wd.v_d[i].im);
        }
    }
    return CUI_OK;
}

uint64_t key_hash(const std::vector<unsigned char>& key) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a, 64 bit
    for (unsigned char c : key) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string cache_path(const char* dir, const std::vector<unsigned char>& key, bool incident_only) {
    char hex[17];
    std::snprintf(hex, sizeof hex, "%016llx", static_cast<unsigned long long>(key_hash(key)));
    std::string path(dir);
    if (!path.empty() && path.back() != '/') path += '/';
    return path + "cui_born_" + hex + (incident_only ? ".incident" : ".tables");
}

cui_status cache_load(const std::string& path, const std::vector<unsigned char>& key, Plan& p, bool* hit) {
    *hit = false;
    File fh;
    fh.f = std::fopen(path.c_str(), "rb");
    if (!fh.f) return CUI_OK;  // no file: compute
    char magic[8];
    uint64_t klen = 0;
    if (std::fread(magic, 1, 8, fh.f) != 8 || std::memcmp(magic, kMagic, 8) != 0 ||
        std::fread(&klen, sizeof klen, 1, fh.f) != 1)
        return set_error(CUI_ERR_INVALID_ARG, "table cache file " + path + " is not a table cache");
    if (klen != key.size())
        return set_error(CUI_ERR_INVALID_ARG, "hash collision: table cache file " + path +
                                                  " was written for a different setup (compute_or_load_hash.m:90-107)");
    std::vector<unsigned char> stored(klen);
    if (std::fread(stored.data(), 1, klen, fh.f) != klen || stored != key)
        return set_error(CUI_ERR_INVALID_ARG, "hash collision: table cache file " + path +
                                                  " was written for a different setup (compute_or_load_hash.m:90-107)");
    Staging stg;
    cudaError_t e = cudaMallocHost(&stg.h, kChunk);
    if (e != cudaSuccess) return check_cuda(e, "cudaMallocHost (table cache)");
    void* dst[2] = {p.table, p.p_in};
    const size_t want[2] = {p.table ? p.table_bytes : 0, p.incident_bytes};  // no table unless stored
    for (int a = 0; a < 2; ++a) {
        uint64_t n = 0;
        if (std::fread(&n, sizeof n, 1, fh.f) != 1 || n != want[a])
            return set_error(CUI_ERR_INVALID_ARG, "table cache file " + path + " is truncated or has other sizes");
        for (size_t off = 0; off < n; off += kChunk) {
            const size_t len = std::min(kChunk, static_cast<size_t>(n) - off);
            if (std::fread(stg.h, 1, len, fh.f) != len)
                return set_error(CUI_ERR_INVALID_ARG, "table cache file " + path + " is truncated");
            if ((e = cudaMemcpy(static_cast<char*>(dst[a]) + off, stg.h, len, cudaMemcpyHostToDevice)) != cudaSuccess)
                return check_cuda(e, "table cache upload");
        }
    }
    *hit = true;
    return CUI_OK;
}

cui_status cache_store(const std::string& path, const std::vector<unsigned char>& key, const Plan& p) {
    const std::string tmp = path + ".tmp";
    Staging stg;
    cudaError_t e = cudaMallocHost(&stg.h, kChunk);
    if (e != cudaSuccess) return check_cuda(e, "cudaMallocHost (table cache)");
    {
        File fh;
        fh.f = std::fopen(tmp.c_str(), "wb");
        if (!fh.f) return set_error(CUI_ERR_INVALID_ARG, "cannot write table cache file " + tmp);
        const uint64_t klen = key.size();
        bool ok = std::fwrite(kMagic, 1, 8, fh.f) == 8 && std::fwrite(&klen, sizeof klen, 1, fh.f) == 1 &&
                  std::fwrite(key.data(), 1, key.size(), fh.f) == key.size();
        const void* src[2] = {p.table, p.p_in};
        const size_t have[2] = {p.table ? p.table_bytes : 0, p.incident_bytes};
        for (int a = 0; a < 2 && ok; ++a) {
            const uint64_t n = have[a];
            ok = std::fwrite(&n, sizeof n, 1, fh.f) == 1;
            for (size_t off = 0; off < n && ok; off += kChunk) {
                const size_t len = std::min(kChunk, static_cast<size_t>(n) - off);
                if ((e = cudaMemcpy(stg.h, static_cast<const char*>(src[a]) + off, len, cudaMemcpyDeviceToHost)) !=
                    cudaSuccess) {
                    std::fclose(fh.f);
                    fh.f = nullptr;
                    std::remove(tmp.c_str());
                    return check_cuda(e, "table cache download");
                }
                ok = std::fwrite(stg.h, 1, len, fh.f) == len;
            }
        }
        ok = (std::fclose(fh.f) == 0) && ok;
        fh.f = nullptr;
        if (!ok) {
            std::remove(tmp.c_str());
            return set_error(CUI_ERR_INVALID_ARG, "writing table cache file " + tmp + " failed");
        }
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        return set_error(CUI_ERR_INVALID_ARG, "cannot rename table cache file into " + path);
    }
    return CUI_OK;
}

}  // namespace cui

extern "C" cui_status cui_born_setup_hash(const cui_born_setup_desc* desc, char* hex17) {
    if (!hex17) return cui::set_error(CUI_ERR_INVALID_ARG, "hex17 is NULL");
    std::vector<unsigned char> key;
    const cui_status s = cui::setup_key(desc, key);
    if (s != CUI_OK) return s;
    std::snprintf(hex17, 17, "%016llx", static_cast<unsigned long long>(cui::key_hash(key)));
    return CUI_OK;
}
