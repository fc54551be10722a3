// File I/O of the C++ host test programs (tests/capi_microiteration.cpp,
// tests/capi_engine.cpp): named arrays written by the Python test and read back.
//
// Format: records of [32-byte name][1-byte type 'i' int32 / 'l' int64 /
// 'd' double][int64 count][count values], little endian.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "qcm_gb300.h"

namespace capi_io {

struct Arr { char type; std::vector<char> bytes; int64_t n; };

inline std::map<std::string, Arr> read_arrays(const char* path) {
    std::map<std::string, Arr> m;
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    char name[32];
    while (std::fread(name, 1, 32, f) == 32) {
        Arr a;
        int64_t n = 0;
        if (std::fread(&a.type, 1, 1, f) != 1 || std::fread(&n, 8, 1, f) != 1) break;
        const size_t w = a.type == 'i' ? 4 : 8;
        a.n = n;
        a.bytes.resize(w * (size_t)n);
        if (n > 0 && std::fread(a.bytes.data(), w, (size_t)n, f) != (size_t)n) throw std::runtime_error("short read");
        m[std::string(name, strnlen(name, 32))] = std::move(a);
    }
    std::fclose(f);
    return m;
}

struct Writer {
    FILE* f;
    explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
        if (!f) throw std::runtime_error(std::string("cannot write ") + path);
    }
    ~Writer() { std::fclose(f); }
    void put(const std::string& name, char type, const void* data, int64_t n) {
        char buf[32] = {0};
        std::strncpy(buf, name.c_str(), 31);
        std::fwrite(buf, 1, 32, f);
        std::fwrite(&type, 1, 1, f);
        std::fwrite(&n, 8, 1, f);
        std::fwrite(data, type == 'i' ? 4 : 8, (size_t)n, f);
    }
};

struct Inputs {
    std::map<std::string, Arr> a;
    template <class T> const T* p(const std::string& k) {
        auto it = a.find(k);
        if (it == a.end()) throw std::runtime_error("missing array " + k);
        return reinterpret_cast<const T*>(it->second.bytes.data());
    }
    int64_t n(const std::string& k) { return a.at(k).n; }
    double d(const std::string& k) { return p<double>(k)[0]; }
    qcm_index_t index(const std::string& k) {
        return {(int32_t)(n(k + ".size")), p<int32_t>(k + ".q"), p<int64_t>(k + ".size")};
    }
    qcm_blocks_t blocks(const std::string& k) {
        return {(int32_t)n(k + ".rows"), p<int32_t>(k + ".q"), p<int64_t>(k + ".rows"), p<int64_t>(k + ".cols"),
                p<int64_t>(k + ".off")};
    }
    qcm_boundary_t boundary(const std::string& k) {
        return {(int32_t)(n(k + ".blk_ptr") - 1), p<int32_t>(k + ".blk_ptr"), p<int32_t>(k + ".q"),
                p<int64_t>(k + ".rows"), p<int64_t>(k + ".cols"), p<int64_t>(k + ".off")};
    }
    qcm_mpo_t mpo(const std::string& k) {
        const int32_t* dims = p<int32_t>(k + ".dims");
        return {dims[0], dims[1], p<int32_t>(k + ".left_spin"), p<int32_t>(k + ".right_spin"),
                p<int32_t>(k + ".left_herm"), p<int32_t>(k + ".right_herm"), p<int32_t>(k + ".left_phase"),
                p<int32_t>(k + ".right_phase"), p<int32_t>(k + ".col_ptr"), p<int32_t>(k + ".row_of"),
                p<int32_t>(k + ".term_ptr"), p<int32_t>(k + ".term_op"), p<double>(k + ".term_scale"), dims[2],
                p<int32_t>(k + ".op_spin"), p<int32_t>(k + ".op_blk_ptr"), p<int32_t>(k + ".blk_q"),
                p<int32_t>(k + ".blk_ent_ptr"), p<int32_t>(k + ".ent"), p<double>(k + ".ent_coeff")};
    }
    double* device(const std::string& k) {
        double* d = nullptr;
        const int64_t len = n(k);
        if (cudaMalloc(&d, sizeof(double) * (len > 0 ? len : 1)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
        if (len > 0) cudaMemcpy(d, p<double>(k), sizeof(double) * len, cudaMemcpyHostToDevice);
        return d;
    }
};

inline void ok(int rc, const char* what) {
    if (rc != QCM_OK) throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) + "): " +
                                               qcm_last_error());
}

}  // namespace capi_io
