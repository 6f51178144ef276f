// Project-written stand-in for the vendored dynamic_bitset, for compiling the
// reference's sources as a test checker.  Same storage layout as
// boost::dynamic_bitset<unsigned long>: bit i lives in block i / 64 at
// position i % 64, unused bits of the last block are zero.  The members the
// reference's BitVectorBuilder / BitVectorIterator reach into (m_bits,
// count_extra_bits, block_index, bit_index) are public here.
#pragma once

#include <climits>
#include <cstddef>
#include <limits>
#include <memory>
#include <string>
#include <vector>

namespace quickfoil {
namespace third_party {
namespace boost {

template <typename Block, typename Allocator>
class dynamic_bitset {
 public:
  typedef std::vector<Block, Allocator> buffer_type;
  typedef Block block_type;
  typedef Allocator allocator_type;
  typedef std::size_t size_type;
  typedef typename buffer_type::size_type block_width_type;
  static constexpr block_width_type bits_per_block = std::numeric_limits<Block>::digits;
  static constexpr size_type npos = static_cast<size_type>(-1);

  dynamic_bitset() : m_num_bits(0) {}
  explicit dynamic_bitset(size_type num_bits) : m_bits(blocks_for(num_bits), Block(0)), m_num_bits(num_bits) {}

  size_type size() const { return m_num_bits; }
  size_type num_blocks() const { return m_bits.size(); }
  bool empty() const { return m_num_bits == 0; }

  void resize(size_type num_bits, bool value = false) {
    const size_type old = m_num_bits;
    m_bits.resize(blocks_for(num_bits), value ? ~Block(0) : Block(0));
    if (value && num_bits > old && old % bits_per_block != 0)
      m_bits[old / bits_per_block] |= ~Block(0) << (old % bits_per_block);
    m_num_bits = num_bits;
    zero_unused_bits();
  }
  void clear() {
    m_bits.clear();
    m_num_bits = 0;
  }
  dynamic_bitset& reset() {
    for (Block& b : m_bits) b = Block(0);
    return *this;
  }
  dynamic_bitset& set() {
    for (Block& b : m_bits) b = ~Block(0);
    zero_unused_bits();
    return *this;
  }
  dynamic_bitset& flip() {
    for (Block& b : m_bits) b = ~b;
    zero_unused_bits();
    return *this;
  }
  dynamic_bitset& set(size_type pos, bool val = true) {
    if (val)
      m_bits[block_index(pos)] |= bit_mask(pos);
    else
      m_bits[block_index(pos)] &= ~bit_mask(pos);
    return *this;
  }
  dynamic_bitset& reset(size_type pos) { return set(pos, false); }
  bool test(size_type pos) const { return (m_bits[block_index(pos)] & bit_mask(pos)) != 0; }
  bool test_set(size_type pos, bool val = true) {
    const bool b = test(pos);
    set(pos, val);
    return b;
  }
  bool operator[](size_type pos) const { return test(pos); }

  size_type count() const {
    size_type c = 0;
    for (Block b : m_bits) c += (size_type)__builtin_popcountll((unsigned long long)b);
    return c;
  }
  bool any() const {
    for (Block b : m_bits)
      if (b) return true;
    return false;
  }
  bool none() const { return !any(); }

  size_type find_first() const { return find_from(0); }
  size_type find_next(size_type pos) const {
    return pos + 1 >= m_num_bits ? npos : find_from(pos + 1);
  }

  dynamic_bitset& operator&=(const dynamic_bitset& o) {
    for (size_type i = 0; i < m_bits.size(); ++i) m_bits[i] &= o.m_bits[i];
    return *this;
  }
  dynamic_bitset& operator|=(const dynamic_bitset& o) {
    for (size_type i = 0; i < m_bits.size(); ++i) m_bits[i] |= o.m_bits[i];
    return *this;
  }
  dynamic_bitset& operator^=(const dynamic_bitset& o) {
    for (size_type i = 0; i < m_bits.size(); ++i) m_bits[i] ^= o.m_bits[i];
    return *this;
  }
  dynamic_bitset operator~() const {
    dynamic_bitset r(*this);
    r.flip();
    return r;
  }
  bool operator==(const dynamic_bitset& o) const {
    return m_num_bits == o.m_num_bits && m_bits == o.m_bits;
  }
  bool operator!=(const dynamic_bitset& o) const { return !(*this == o); }

  block_width_type count_extra_bits() const { return bit_index(size()); }
  static size_type block_index(size_type pos) { return pos / bits_per_block; }
  static block_width_type bit_index(size_type pos) {
    return static_cast<block_width_type>(pos % bits_per_block);
  }

  buffer_type m_bits;
  size_type m_num_bits;

 private:
  static size_type blocks_for(size_type n) { return (n + bits_per_block - 1) / bits_per_block; }
  static Block bit_mask(size_type pos) { return Block(1) << bit_index(pos); }
  void zero_unused_bits() {
    const block_width_type extra = count_extra_bits();
    if (extra != 0) m_bits.back() &= ~(~Block(0) << extra);
  }
  size_type find_from(size_type pos) const {
    size_type blk = block_index(pos);
    if (blk >= m_bits.size()) return npos;
    Block cur = m_bits[blk] & (~Block(0) << bit_index(pos));
    while (true) {
      if (cur) return blk * bits_per_block + (size_type)__builtin_ctzll((unsigned long long)cur);
      if (++blk >= m_bits.size()) return npos;
      cur = m_bits[blk];
    }
  }
};

template <typename B, typename A>
dynamic_bitset<B, A> operator&(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) {
  dynamic_bitset<B, A> r(x);
  return r &= y;
}
template <typename B, typename A>
dynamic_bitset<B, A> operator|(const dynamic_bitset<B, A>& x, const dynamic_bitset<B, A>& y) {
  dynamic_bitset<B, A> r(x);
  return r |= y;
}

// Most significant bit first, as boost::to_string writes it.
template <typename B, typename A>
void to_string(const dynamic_bitset<B, A>& b, std::string& s) {
  s.assign(b.size(), '0');
  for (std::size_t i = 0; i < b.size(); ++i)
    if (b.test(i)) s[b.size() - 1 - i] = '1';
}

}  // namespace boost
}  // namespace third_party
}  // namespace quickfoil
