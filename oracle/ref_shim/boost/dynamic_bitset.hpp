/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The members of boost::dynamic_bitset<> that the reference simulator uses for
 * its synapse indicators (c++/include/NetworkGrowthSimulator.h:22, 170-172):
 * resize (new bits clear), reset (clear all), size and element access that can
 * be assigned 0/1 and compared with 0/1.  One byte per bit: the indicator
 * rows are small and byte access keeps the shim simple.
 */
#ifndef UG_REF_SHIM_DYNAMIC_BITSET_HPP
#define UG_REF_SHIM_DYNAMIC_BITSET_HPP

#include <algorithm>
#include <cstddef>
#include <vector>

namespace boost {

template <class Block = unsigned long>
class dynamic_bitset {
public:
    typedef std::size_t size_type;

    class reference {
    public:
        explicit reference(unsigned char& b) : b_(b) {}
        reference& operator=(bool v) { b_ = v ? 1 : 0; return *this; }
        reference& operator=(const reference& o) { b_ = o.b_; return *this; }
        operator bool() const { return b_ != 0; }
        bool operator~() const { return b_ == 0; }

    private:
        unsigned char& b_;
    };

    dynamic_bitset() {}
    explicit dynamic_bitset(size_type n) : bits_(n, 0) {}

    void resize(size_type n, bool value = false) { bits_.resize(n, value ? 1 : 0); }
    size_type size() const { return bits_.size(); }
    dynamic_bitset& reset() { std::fill(bits_.begin(), bits_.end(), 0); return *this; }
    dynamic_bitset& reset(size_type i) { bits_[i] = 0; return *this; }
    dynamic_bitset& set(size_type i, bool v = true) { bits_[i] = v ? 1 : 0; return *this; }
    bool test(size_type i) const { return bits_[i] != 0; }
    size_type count() const { return (size_type)std::count(bits_.begin(), bits_.end(), 1); }

    reference operator[](size_type i) { return reference(bits_[i]); }
    bool operator[](size_type i) const { return bits_[i] != 0; }

private:
    std::vector<unsigned char> bits_;
};

} // namespace boost

#endif
