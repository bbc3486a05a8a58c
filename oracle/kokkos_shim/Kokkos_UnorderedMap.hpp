// Serial Kokkos-subset shim (test infrastructure only): a linear-probing set
// with the UnorderedMap calls made by ExaMiniMD's NeighborCSRMapConstr
// (src/neighbor_types/neighbor_csr_map_constr.h:101-320).  That module is out
// of the hot-path scope; this exists so the reference translation units that
// include it compile and link.
#ifndef EMD_KOKKOS_SHIM_UMAP_HPP
#define EMD_KOKKOS_SHIM_UMAP_HPP
#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class Key, class Value = void, class Device = void, class Hasher = void, class EqualTo = void>
class UnorderedMap {
  struct Store {
    std::vector<Key> keys;
    std::vector<char> used;
    size_t count = 0;
    bool failed = false;
  };
  std::shared_ptr<Store> s_;
  static size_t hash(const Key& k) {
    const unsigned long long a = (unsigned long long)(unsigned)k.first;
    const unsigned long long b = (unsigned long long)(unsigned)k.second;
    return size_t((a * 0x9E3779B97F4A7C15ull) ^ (b + 0x632BE59BD9B4E019ull + (a << 6)));
  }

 public:
  struct insert_result {
    bool ok, existed, fail;
    bool success() const { return ok; }
    bool existing() const { return existed; }
    bool failed() const { return fail; }
  };
  explicit UnorderedMap(size_t capacity = 0) : s_(std::make_shared<Store>()) { rehash(capacity); }
  insert_result insert(const Key& k) const {
    Store& s = *s_;
    const size_t cap = s.keys.size();
    if (cap == 0) { s.failed = true; return {false, false, true}; }
    size_t h = hash(k) % cap;
    for (size_t probe = 0; probe < cap; ++probe) {
      const size_t slot = (h + probe) % cap;
      if (!s.used[slot]) {
        s.used[slot] = 1;
        s.keys[slot] = k;
        ++s.count;
        return {true, false, false};
      }
      if (s.keys[slot] == k) return {false, true, false};
    }
    s.failed = true;
    return {false, false, true};
  }
  bool valid_at(size_t i) const { return s_->used[i] != 0; }
  Key key_at(size_t i) const { return s_->keys[i]; }
  size_t capacity() const { return s_->keys.size(); }
  size_t size() const { return s_->count; }
  bool failed_insert() const { return s_->failed; }
  void clear() {
    std::fill(s_->used.begin(), s_->used.end(), 0);
    s_->count = 0;
    s_->failed = false;
  }
  bool rehash(size_t n) {
    if (!s_) s_ = std::make_shared<Store>();
    std::vector<Key> old_keys = s_->keys;
    std::vector<char> old_used = s_->used;
    s_->keys.assign(n, Key());
    s_->used.assign(n, 0);
    s_->count = 0;
    s_->failed = false;
    for (size_t i = 0; i < old_keys.size(); ++i)
      if (old_used[i]) insert(old_keys[i]);
    return true;
  }
};
}  // namespace Kokkos
#endif
