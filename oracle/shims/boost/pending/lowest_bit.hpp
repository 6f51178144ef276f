// Shim for boost::lowest_bit: index of the least significant set bit.
#pragma once
namespace boost {
template <class T>
inline int lowest_bit(T x) { return __builtin_ctzll(static_cast<unsigned long long>(x)); }
}  // namespace boost
