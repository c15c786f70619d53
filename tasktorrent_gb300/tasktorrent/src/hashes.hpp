// Hash for task keys (int or std::array<int,N>), used by Taskflow's
// dependency map.  The reference uses FNV-1a over the key bytes
// (tasktorrent/src/hashes.hpp:44-57); any good hash gives the same
// behaviour, this one is FNV-1a over the key's integers.
#ifndef TTOR_GB300_HASHES_HPP
#define TTOR_GB300_HASHES_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>

namespace ttor {

template <class T>
struct hash_int_N {
    size_t operator()(const T& t) const { return std::hash<T>{}(t); }
};

template <class T, std::size_t N>
struct hash_int_N<std::array<T, N>> {
    size_t operator()(const std::array<T, N>& t) const {
        uint64_t h = 0xcbf29ce484222325ULL;
        for (std::size_t i = 0; i < N; ++i) h = (h ^ (uint64_t)(uint32_t)t[i]) * 0x100000001b3ULL;
        return (size_t)h;
    }
};

}  // namespace ttor

#endif
