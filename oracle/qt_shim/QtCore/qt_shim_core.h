// qt_shim_core.h -- the few QtCore containers that the reference's
// downsample.cpp and the headers of its CUDA code use (QVector, QList,
// QHash, QMap and their Java-style iterators), over the standard library, plus empty QString / QStringList /
// QFile types that its headers name, so that those files compile for the
// oracle's reference checks without Qt.  Test infrastructure only.
//
// Semantics kept: QVector(n) value-initialises; insert() on QHash/QMap
// replaces the value of an existing key; QMapIterator walks keys in
// ascending order.  QHash iteration order is unspecified in Qt (seeded per
// process); here it is descending key order, one of the orders Qt may give
// (with it, downsampleVote's ties go to the smallest value).
#pragma once
#include <map>
#include <vector>

#ifndef Q_UNUSED
#define Q_UNUSED(x) (void)(x)
#endif

template <class T>
class QVector {
public:
    QVector() {}
    explicit QVector(int n) : v_(n < 0 ? 0 : (size_t)n, T()) {}
    QVector(const QVector& o) : v_(o.v_) {}
    QVector& operator=(const QVector& o) { v_ = o.v_; return *this; }
    T* data() { return v_.data(); }
    const T* data() const { return v_.data(); }
    const T* constData() const { return v_.data(); }
    int size() const { return (int)v_.size(); }
    T& operator[](int i) { return v_[(size_t)i]; }
    const T& operator[](int i) const { return v_[(size_t)i]; }
    void resize(int n) { v_.resize((size_t)n); }
    void append(const T& t) { v_.push_back(t); }
    bool isEmpty() const { return v_.empty(); }
    const T& at(int i) const { return v_[(size_t)i]; }
    void clear() { v_.clear(); }

private:
    std::vector<T> v_;
};

template <class T>
class QList {
public:
    void append(const T& t) { v_.push_back(t); }
    T& last() { return v_.back(); }
    const T& last() const { return v_.back(); }
    int size() const { return (int)v_.size(); }
    T& operator[](int i) { return v_[(size_t)i]; }
    const T& operator[](int i) const { return v_[(size_t)i]; }
    const T& at(int i) const { return v_[(size_t)i]; }
    void clear() { v_.clear(); }
    bool isEmpty() const { return v_.empty(); }
    T& first() { return v_.front(); }
    const T& first() const { return v_.front(); }
    void push_front(const T& t) { v_.insert(v_.begin(), t); }
    T takeLast() { T t = v_.back(); v_.pop_back(); return t; }

private:
    std::vector<T> v_;
};

// Declaration-level stand-ins: the reference's headers name these types in
// signatures and members; nothing here calls into them.
class QString {
public:
    QString() {}
    QString(const char*) {}
};
class QStringList : public QList<QString> {};
class QFile {};

template <class K, class V>
class QHash {
public:
    void insert(const K& k, const V& v) { m_[k] = v; }
    V value(const K& k, const V& dflt) const {
        typename std::map<K, V>::const_iterator it = m_.find(k);
        return it == m_.end() ? dflt : it->second;
    }
    const std::map<K, V>& items() const { return m_; }

private:
    std::map<K, V> m_;
};

template <class K, class V>
class QHashIterator {
public:
    explicit QHashIterator(const QHash<K, V>& h) : m_(h.items()), it_(m_.rbegin()), cur_(m_.rend()) {}
    bool hasNext() const { return it_ != m_.rend(); }
    void next() { cur_ = it_++; }
    const K& key() const { return cur_->first; }
    const V& value() const { return cur_->second; }

private:
    const std::map<K, V>& m_;
    typename std::map<K, V>::const_reverse_iterator it_, cur_;
};

template <class K, class V>
class QMap {
public:
    void insert(const K& k, const V& v) { m_[k] = v; }
    const std::map<K, V>& items() const { return m_; }

private:
    std::map<K, V> m_;
};

template <class K, class V>
class QMapIterator {
public:
    struct Item {
        typename std::map<K, V>::const_iterator it;
        const K& key() const { return it->first; }
        const V& value() const { return it->second; }
    };
    explicit QMapIterator(const QMap<K, V>& m) : m_(m.items()), it_(m_.begin()) {}
    void toBack() { it_ = m_.end(); }
    bool hasPrevious() const { return it_ != m_.begin(); }
    Item previous() { Item r; r.it = --it_; return r; }

private:
    const std::map<K, V>& m_;
    typename std::map<K, V>::const_iterator it_;
};
