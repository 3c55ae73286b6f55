/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The members of boost::circular_buffer that the reference simulator uses
 * (c++/include/NetworkGrowthSimulator.h:21 and its activity history):
 * construction with a capacity, push_front / push_back that overwrite the far
 * end once the buffer is full, indexing from the front, size, and begin/end
 * iterators that can be read and written.  After push_back has filled an
 * empty buffer its elements are stored in index order, so &buf[0] addresses
 * them contiguously, as boost's does in the same state.
 */
#ifndef UG_REF_SHIM_CIRCULAR_BUFFER_HPP
#define UG_REF_SHIM_CIRCULAR_BUFFER_HPP

#include <cstddef>
#include <iterator>
#include <vector>

namespace boost {

template <class T>
class circular_buffer {
public:
    typedef T value_type;
    typedef std::size_t size_type;
    typedef std::ptrdiff_t difference_type;
    typedef T& reference;
    typedef const T& const_reference;

    template <class Owner, class Ref, class Ptr>
    class iter_base {
    public:
        typedef std::random_access_iterator_tag iterator_category;
        typedef T value_type;
        typedef std::ptrdiff_t difference_type;
        typedef Ptr pointer;
        typedef Ref reference;

        iter_base() : b_(nullptr), i_(0) {}
        iter_base(Owner* b, std::size_t i) : b_(b), i_(i) {}
        Ref operator*() const { return (*b_)[i_]; }
        Ptr operator->() const { return &(*b_)[i_]; }
        Ref operator[](difference_type k) const { return (*b_)[i_ + k]; }
        iter_base& operator++() { ++i_; return *this; }
        iter_base operator++(int) { iter_base t = *this; ++i_; return t; }
        iter_base& operator--() { --i_; return *this; }
        iter_base operator--(int) { iter_base t = *this; --i_; return t; }
        iter_base& operator+=(difference_type k) { i_ += k; return *this; }
        iter_base& operator-=(difference_type k) { i_ -= k; return *this; }
        iter_base operator+(difference_type k) const { return iter_base(b_, i_ + k); }
        iter_base operator-(difference_type k) const { return iter_base(b_, i_ - k); }
        difference_type operator-(const iter_base& o) const { return (difference_type)i_ - (difference_type)o.i_; }
        bool operator==(const iter_base& o) const { return i_ == o.i_; }
        bool operator!=(const iter_base& o) const { return i_ != o.i_; }
        bool operator<(const iter_base& o) const { return i_ < o.i_; }
        bool operator>(const iter_base& o) const { return i_ > o.i_; }
        bool operator<=(const iter_base& o) const { return i_ <= o.i_; }
        bool operator>=(const iter_base& o) const { return i_ >= o.i_; }

    private:
        Owner* b_;
        std::size_t i_;
    };

    typedef iter_base<circular_buffer, T&, T*> iterator;
    typedef iter_base<const circular_buffer, const T&, const T*> const_iterator;

    circular_buffer() : first_(0), size_(0) {}
    explicit circular_buffer(size_type capacity) : store_(capacity), first_(0), size_(0) {}

    size_type capacity() const { return store_.size(); }
    size_type size() const { return size_; }
    bool empty() const { return size_ == 0; }
    bool full() const { return size_ == store_.size(); }
    void clear() { first_ = 0; size_ = 0; }

    T& operator[](size_type i) { return store_[(first_ + i) % store_.size()]; }
    const T& operator[](size_type i) const { return store_[(first_ + i) % store_.size()]; }
    T& front() { return (*this)[0]; }
    T& back() { return (*this)[size_ - 1]; }

    void push_back(const T& x)
    {
        if (store_.empty()) return;
        if (full()) {
            store_[first_] = x;  /* the new last element replaces the first */
            first_ = (first_ + 1) % store_.size();
        } else {
            store_[(first_ + size_) % store_.size()] = x;
            ++size_;
        }
    }

    void push_front(const T& x)
    {
        if (store_.empty()) return;
        first_ = (first_ + store_.size() - 1) % store_.size();
        store_[first_] = x;      /* when full this overwrites the old last element */
        if (!full()) ++size_;
    }

    iterator begin() { return iterator(this, 0); }
    iterator end() { return iterator(this, size_); }
    const_iterator begin() const { return const_iterator(this, 0); }
    const_iterator end() const { return const_iterator(this, size_); }

private:
    std::vector<T> store_;
    size_type first_;
    size_type size_;
};

} // namespace boost

#endif
