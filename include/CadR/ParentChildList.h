// CadR/ParentChildList.h - parent/child relations between objects of one
// type, with the interface of the reference's src/CadR/ParentChildList.h:
// a type T holds a ChildList<T, offsets> and a ParentList<T, offsets>
// member, and `offsets` (a static ParentChildListOffsets of T) tells where
// both members lie inside T.
//
// Each relation is one node linked into two lists at once: the parent's
// child list and the child's parent list.  append() on either side links
// the node into both, remove() on either side unlinks it from both and
// frees it, clear() removes every relation of the list, and a list's
// destructor clears it, so destroying an object detaches it from all its
// parents and children.  Iterators are bidirectional and yield the child
// (ChildList) or the parent (ParentList).
//
// Difference from the reference: ParentList::front() and back() return the
// first and last parent; the reference's return the list's owner.
#pragma once

#include <cstddef>
#include <iterator>
#include <type_traits>

namespace CadR {

struct ParentChildListOffsets {
    size_t parentListOffset;  // offset of T's ParentList member inside T
    size_t childListOffset;   // offset of T's ChildList member inside T
};

template <typename Type>
struct ParentChildRelation {
    ParentChildRelation* prevInParent = nullptr;  // links of the parent's child list
    ParentChildRelation* nextInParent = nullptr;
    ParentChildRelation* prevInChild = nullptr;   // links of the child's parent list
    ParentChildRelation* nextInChild = nullptr;
    Type* child = nullptr;
    Type* parent = nullptr;
};

template <typename Type, const ParentChildListOffsets& listOffsets>
class ParentList;
template <typename Type, const ParentChildListOffsets& listOffsets>
class ChildList;

namespace detail {

// A circular list of relation nodes through one pair of their links, with
// a sentinel node of its own.
template <typename Type, bool kParentSide>
class RelationRing {
public:
    using Node = ParentChildRelation<Type>;

    RelationRing() { prev(&_head) = next(&_head) = &_head; }
    RelationRing(const RelationRing&) = delete;
    RelationRing& operator=(const RelationRing&) = delete;

    static Node*& prev(Node* n) { return kParentSide ? n->prevInParent : n->prevInChild; }
    static Node*& next(Node* n) { return kParentSide ? n->nextInParent : n->nextInChild; }
    Node* sentinel() const { return const_cast<Node*>(&_head); }
    Node* first() const { return next(sentinel()); }
    Node* last() const { return prev(sentinel()); }
    bool empty() const { return first() == sentinel(); }
    size_t size() const
    {
        size_t k = 0;
        for (Node* n = first(); n != sentinel(); n = next(n)) k++;
        return k;
    }
    void pushBack(Node* n)
    {
        Node* l = last();
        prev(n) = l;
        next(n) = sentinel();
        next(l) = n;
        prev(sentinel()) = n;
    }
    static void unlink(Node* n)
    {
        next(prev(n)) = next(n);
        prev(next(n)) = prev(n);
        prev(n) = next(n) = nullptr;
    }

private:
    Node _head;
};

}  // namespace detail

// Iterator over one side's ring.  kParentSide: the ring of a ChildList (its
// nodes yield children); kYieldChild: what operator* returns.
template <typename Type, bool kParentSide, bool kYieldChild, bool kReverse, bool kConst>
class ParentChildIterator {
    using Node = ParentChildRelation<Type>;
    using Ring = detail::RelationRing<Type, kParentSide>;
    Node* _n = nullptr;

public:
    using iterator_category = std::bidirectional_iterator_tag;
    using value_type = Type;
    using difference_type = std::ptrdiff_t;
    using reference = typename std::conditional<kConst, const Type&, Type&>::type;
    using pointer = typename std::conditional<kConst, const Type*, Type*>::type;

    ParentChildIterator() = default;
    explicit ParentChildIterator(Node* n) : _n(n) {}
    // iterator -> const_iterator
    template <bool C = kConst, typename = typename std::enable_if<C>::type>
    ParentChildIterator(const ParentChildIterator<Type, kParentSide, kYieldChild, kReverse, false>& o)
        : _n(o.node())
    {
    }

    Node* node() const { return _n; }
    reference operator*() const { return kYieldChild ? *_n->child : *_n->parent; }
    pointer operator->() const { return kYieldChild ? _n->child : _n->parent; }
    ParentChildIterator& operator++()
    {
        _n = kReverse ? Ring::prev(_n) : Ring::next(_n);
        return *this;
    }
    ParentChildIterator operator++(int)
    {
        ParentChildIterator t = *this;
        ++*this;
        return t;
    }
    ParentChildIterator& operator--()
    {
        _n = kReverse ? Ring::next(_n) : Ring::prev(_n);
        return *this;
    }
    ParentChildIterator operator--(int)
    {
        ParentChildIterator t = *this;
        --*this;
        return t;
    }
    bool operator==(const ParentChildIterator& o) const { return _n == o._n; }
    bool operator!=(const ParentChildIterator& o) const { return _n != o._n; }
};

// The children of the object that holds this list.
template <typename Type, const ParentChildListOffsets& listOffsets>
class ChildList {
    using Node = ParentChildRelation<Type>;
    using Ring = detail::RelationRing<Type, true>;

public:
    using iterator = ParentChildIterator<Type, true, true, false, false>;
    using const_iterator = ParentChildIterator<Type, true, true, false, true>;
    using reverse_iterator = ParentChildIterator<Type, true, true, true, false>;
    using const_reverse_iterator = ParentChildIterator<Type, true, true, true, true>;

    ChildList() = default;
    ChildList(const ChildList&) = delete;
    ChildList& operator=(const ChildList&) = delete;
    ~ChildList() { clear(); }

    Type& front() { return *_ring.first()->child; }
    const Type& front() const { return *_ring.first()->child; }
    Type& back() { return *_ring.last()->child; }
    const Type& back() const { return *_ring.last()->child; }
    iterator begin() { return iterator(_ring.first()); }
    const_iterator begin() const { return const_iterator(_ring.first()); }
    const_iterator cbegin() const { return begin(); }
    iterator end() { return iterator(_ring.sentinel()); }
    const_iterator end() const { return const_iterator(_ring.sentinel()); }
    const_iterator cend() const { return end(); }
    reverse_iterator rbegin() { return reverse_iterator(_ring.last()); }
    const_reverse_iterator rbegin() const { return const_reverse_iterator(_ring.last()); }
    const_reverse_iterator crbegin() const { return rbegin(); }
    reverse_iterator rend() { return reverse_iterator(_ring.sentinel()); }
    const_reverse_iterator rend() const { return const_reverse_iterator(_ring.sentinel()); }
    const_reverse_iterator crend() const { return rend(); }
    size_t size() const { return _ring.size(); }
    bool empty() const { return _ring.empty(); }

    // Makes `child` the last child of this list's owner (and the owner the
    // last parent of `child`).
    iterator append(Type& child)
    {
        Node* r = new Node;
        r->child = &child;
        r->parent = owner();
        _ring.pushBack(r);
        ParentList<Type, listOffsets>::of(child)._ring.pushBack(r);
        return iterator(r);
    }
    // Removes the relation `it` points at, from both lists.
    void remove(iterator it)
    {
        Node* r = it.node();
        Ring::unlink(r);
        detail::RelationRing<Type, false>::unlink(r);
        delete r;
    }
    void clear()
    {
        while (!empty()) remove(begin());
    }

    static ChildList& of(Type& t)
    {
        return *reinterpret_cast<ChildList*>(reinterpret_cast<char*>(&t) + listOffsets.childListOffset);
    }

private:
    Type* owner() { return reinterpret_cast<Type*>(reinterpret_cast<char*>(this) - listOffsets.childListOffset); }
    Ring _ring;
    friend class ParentList<Type, listOffsets>;
};

// The parents of the object that holds this list.
template <typename Type, const ParentChildListOffsets& listOffsets>
class ParentList {
    using Node = ParentChildRelation<Type>;
    using Ring = detail::RelationRing<Type, false>;

public:
    using iterator = ParentChildIterator<Type, false, false, false, false>;
    using const_iterator = ParentChildIterator<Type, false, false, false, true>;
    using reverse_iterator = ParentChildIterator<Type, false, false, true, false>;
    using const_reverse_iterator = ParentChildIterator<Type, false, false, true, true>;

    ParentList() = default;
    ParentList(const ParentList&) = delete;
    ParentList& operator=(const ParentList&) = delete;
    ~ParentList() { clear(); }

    Type& front() { return *_ring.first()->parent; }
    const Type& front() const { return *_ring.first()->parent; }
    Type& back() { return *_ring.last()->parent; }
    const Type& back() const { return *_ring.last()->parent; }
    iterator begin() { return iterator(_ring.first()); }
    const_iterator begin() const { return const_iterator(_ring.first()); }
    const_iterator cbegin() const { return begin(); }
    iterator end() { return iterator(_ring.sentinel()); }
    const_iterator end() const { return const_iterator(_ring.sentinel()); }
    const_iterator cend() const { return end(); }
    reverse_iterator rbegin() { return reverse_iterator(_ring.last()); }
    const_reverse_iterator rbegin() const { return const_reverse_iterator(_ring.last()); }
    const_reverse_iterator crbegin() const { return rbegin(); }
    reverse_iterator rend() { return reverse_iterator(_ring.sentinel()); }
    const_reverse_iterator rend() const { return const_reverse_iterator(_ring.sentinel()); }
    const_reverse_iterator crend() const { return rend(); }
    size_t size() const { return _ring.size(); }
    bool empty() const { return _ring.empty(); }

    // Makes `parent` the last parent of this list's owner (and the owner the
    // last child of `parent`).
    iterator append(Type& parent)
    {
        Node* r = new Node;
        r->child = owner();
        r->parent = &parent;
        ChildList<Type, listOffsets>::of(parent)._ring.pushBack(r);
        _ring.pushBack(r);
        return iterator(r);
    }
    // Removes the relation `it` points at, from both lists.
    void remove(iterator it)
    {
        Node* r = it.node();
        Ring::unlink(r);
        detail::RelationRing<Type, true>::unlink(r);
        delete r;
    }
    void clear()
    {
        while (!empty()) remove(begin());
    }

    static ParentList& of(Type& t)
    {
        return *reinterpret_cast<ParentList*>(reinterpret_cast<char*>(&t) + listOffsets.parentListOffset);
    }

private:
    Type* owner() { return reinterpret_cast<Type*>(reinterpret_cast<char*>(this) - listOffsets.parentListOffset); }
    Ring _ring;
    friend class ChildList<Type, listOffsets>;
};

}  // namespace CadR
