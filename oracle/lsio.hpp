// Lattice case files: a flat list of named, typed arrays.
//
// Test infrastructure only. One record is
//   u32 name_length | name bytes | u8 type code | u64 element count | raw little-endian data
// with type codes 'd' (f64), 'f' (f32), 'I' (u32), 'Q' (u64), 'B' (u8). The same
// files carry the inputs of a lattice case (positions, bonds, settings) to the
// reference harness, to the CPU restatement and to the GPU tests, and carry
// their outputs back, so every checker reads exactly the same bytes.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace lsio {

struct Array {
    char type{'B'};
    std::vector<unsigned char> bytes;
    [[nodiscard]] std::size_t width() const {
        switch (type) {
        case 'd': case 'Q': return 8;
        case 'f': case 'I': return 4;
        default: return 1;
        }
    }
    [[nodiscard]] std::size_t count() const { return bytes.size() / width(); }
};

class Case {
public:
    std::map<std::string, Array> arrays;

    [[nodiscard]] bool has(const std::string &name) const { return arrays.count(name) != 0; }

    template <typename T>
    [[nodiscard]] std::vector<T> get(const std::string &name) const {
        const auto it = arrays.find(name);
        if (it == arrays.end()) throw std::runtime_error("case has no array '" + name + "'");
        const Array &a = it->second;
        if (a.width() != sizeof(T)) throw std::runtime_error("array '" + name + "' has another element width");
        std::vector<T> out(a.count());
        if (!out.empty()) std::memcpy(out.data(), a.bytes.data(), a.bytes.size());
        return out;
    }
    template <typename T>
    [[nodiscard]] T scalar(const std::string &name) const {
        const auto v = get<T>(name);
        if (v.size() != 1) throw std::runtime_error("array '" + name + "' is not a scalar");
        return v[0];
    }
    template <typename T>
    [[nodiscard]] T scalarOr(const std::string &name, T fallback) const {
        return has(name) ? scalar<T>(name) : fallback;
    }

    template <typename T>
    void put(const std::string &name, const std::vector<T> &values) {
        Array a;
        a.type = typeCode<T>();
        a.bytes.resize(values.size() * sizeof(T));
        if (!values.empty()) std::memcpy(a.bytes.data(), values.data(), a.bytes.size());
        arrays[name] = std::move(a);
    }
    template <typename T>
    void putScalar(const std::string &name, T value) { put<T>(name, std::vector<T>{value}); }

    void read(const std::string &path) {
        FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + path);
        arrays.clear();
        for (;;) {
            std::uint32_t len = 0;
            if (std::fread(&len, 4, 1, f) != 1) break;
            std::string name(len, '\0');
            char type = 0;
            std::uint64_t count = 0;
            if (std::fread(name.data(), 1, len, f) != len || std::fread(&type, 1, 1, f) != 1 ||
                std::fread(&count, 8, 1, f) != 1) {
                std::fclose(f);
                throw std::runtime_error("truncated case file " + path);
            }
            Array a;
            a.type = type;
            a.bytes.resize(count * a.width());
            if (count && std::fread(a.bytes.data(), 1, a.bytes.size(), f) != a.bytes.size()) {
                std::fclose(f);
                throw std::runtime_error("truncated case file " + path);
            }
            arrays[name] = std::move(a);
        }
        std::fclose(f);
    }

    void write(const std::string &path) const {
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) throw std::runtime_error("cannot write " + path);
        for (const auto &[name, a] : arrays) {
            const std::uint32_t len = static_cast<std::uint32_t>(name.size());
            const std::uint64_t count = a.count();
            std::fwrite(&len, 4, 1, f);
            std::fwrite(name.data(), 1, len, f);
            std::fwrite(&a.type, 1, 1, f);
            std::fwrite(&count, 8, 1, f);
            if (!a.bytes.empty()) std::fwrite(a.bytes.data(), 1, a.bytes.size(), f);
        }
        std::fclose(f);
    }

private:
    template <typename T> static char typeCode();
};

template <> inline char Case::typeCode<double>() { return 'd'; }
template <> inline char Case::typeCode<float>() { return 'f'; }
template <> inline char Case::typeCode<std::uint32_t>() { return 'I'; }
template <> inline char Case::typeCode<std::uint64_t>() { return 'Q'; }
template <> inline char Case::typeCode<std::uint8_t>() { return 'B'; }

} // namespace lsio
