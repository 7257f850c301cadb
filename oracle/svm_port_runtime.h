/*
 * ORACLE (test infrastructure only).  A restatement of the runtime that the
 * reference's generated host code links against: the columnar Bulk layout
 * (com/cpp/define.hpp:15-87), BulkVector (com/cpp/cpu-runtime.hpp:13-32), the
 * byte-polynomial Hash (cpu-runtime.hpp:68-74), capped linear-probing insert
 * (cpu-runtime.hpp:80-91) and probe (cpu-runtime.hpp:125-138).
 *
 * The same generated query text (oracle/codegen.py) compiles against this
 * header or against the reference's own headers (oracle/_ref); the two builds
 * are compared by the oracle tests.
 *
 * Signedness: the reference hashes and compares key bytes through plain
 * `char`, which is signed on x86 and unsigned on aarch64.  This header fixes
 * the x86 behaviour (signed) on every host, for Hash and StrCmp alike; define
 * SVM_PORT_UNSIGNED_CHAR to get the aarch64 one.
 */
#ifndef SVM_PORT_RUNTIME_H_
#define SVM_PORT_RUNTIME_H_

#include <stddef.h>
#include <stdint.h>

typedef unsigned long long uint64;

/* define.hpp:17-29 */
const uint64 KB = 1024;
const uint64 MB = 1024 * 1024;
const uint64 PageSize = 4 * KB;
const uint64 MaxColumnNum = 24;
const uint64 MaxDim = 32;
const uint64 MaxBulkInputNum = 8;
const uint64 HashRate = 5;

#ifdef SVM_PORT_UNSIGNED_CHAR
typedef unsigned char svm_hash_byte;
#else
typedef signed char svm_hash_byte;
#endif

/* define.hpp:43-58: column types and sizes of one bulk. */
class Schema {
 public:
  int column_type_[MaxColumnNum];
  uint64 column_size_[MaxColumnNum];
  uint64 column_ct_ = 0;
  void AddColumn(int type, uint64 size) {
    column_type_[column_ct_] = type;
    column_size_[column_ct_] = size;
    column_ct_++;
  }
  uint64 GetColumnSize(uint64 c) const { return column_size_[c]; }
  uint64 GetColumnCount() const { return column_ct_; }
};

/* define.hpp:69-87: one buffer holding every column of a row range. */
class Bulk {
 public:
  void SetColumnPos(uint64 col, uint64 offset) { column_pos_[col] = offset; }
  void Init(void* buffer, uint64 capacity) {
    buffer_ = buffer;
    capacity_ = capacity;
    for (uint64 c = 0; c < schema_.GetColumnCount(); c++)
      column_buf_[c] = (char*)buffer_ + column_pos_[c];
  }
  uint64 id_ = 0;
  uint64 capacity_ = 0;
  uint64 tuple_count_ = 0;
  uint64 max_tuple_count_ = 0;
  uint64 column_pos_[MaxColumnNum];
  void* column_buf_[MaxColumnNum];
  Schema schema_;
  void* buffer_ = nullptr;
};

/* cpu-runtime.hpp:13-32: the column pointers of the fact bulk (slot 0) and of
 * bulk 0 of every joined object (slots 1..), passed by value to the query. */
class BulkVector {
 public:
  BulkVector() {}
  explicit BulkVector(Bulk* b) { AddBulk(b); }
  inline void* GetColumn(int obj, int col) { return buffer_[obj][col]; }
  uint64 GetTupleCount() { return tuple_ct_[0]; }
  void AddBulk(Bulk* b) {
    for (uint64 c = 0; c < b->schema_.column_ct_; c++) buffer_[bulk_ct_][c] = b->column_buf_[c];
    tuple_ct_[bulk_ct_] = b->tuple_count_;
    max_tuple_ct_[bulk_ct_] = b->max_tuple_count_;
    bulk_ct_++;
  }
  uint64 bulk_ct_ = 0;
  void* buffer_[MaxBulkInputNum][MaxColumnNum];
  uint64 tuple_ct_[MaxBulkInputNum];
  uint64 max_tuple_ct_[MaxBulkInputNum];
};

/* cpu-runtime.hpp:68-74: h = h*31 + byte over n bytes, then clear bit 31. */
inline unsigned Hash(const char* p, int n) {
  const svm_hash_byte* b = (const svm_hash_byte*)p;
  unsigned h = 0;
  for (int k = 0; k < n; k++) h = h * 31u + (unsigned)(int)b[k];
  return h & 0x7FFFFFFFu;
}

/* cpu-runtime.hpp:37-44: compare at most n bytes, stopping at either NUL;
 * the difference of the first unequal bytes, as chars of the same
 * signedness as Hash's. */
inline int StrCmp(const char* a, const char* b, int n) {
  const svm_hash_byte* x = (const svm_hash_byte*)a;
  const svm_hash_byte* y = (const svm_hash_byte*)b;
  for (int k = 0; k < n; k++) {
    if (x[k] == 0 || y[k] == 0) return 0;
    if (x[k] != y[k]) return (int)x[k] - (int)y[k];
  }
  return 0;
}

inline void StrCopy(char* d, char* s, int n) {
  for (int k = 0; k < n; k++) d[k] = s[k];
}

/* cpu-runtime.hpp:80-91: place row `pos` in the first free slot (-1) among
 * the 10 slots starting at its home slot; give up after 10. */
template <typename T>
inline bool InsertHashTable(T* tab, int pos, unsigned key_size, int* ht, unsigned ht_size) {
  unsigned slot = Hash((const char*)(tab + pos), key_size) % ht_size;
  for (int step = 0; step < 10; step++) {
    if (ht[slot] < 0) {
      ht[slot] = pos;
      return true;
    }
    slot = (slot + 1) % ht_size;
  }
  return false;
}

/* cpu-runtime.hpp:125-138: walk at most 10 slots from the key's home slot;
 * stop at an empty slot; return the first row whose key equals *key. */
template <typename T>
inline int Probe(T* key, unsigned key_size, T* tab, int* ht, unsigned ht_size) {
  unsigned slot = Hash((const char*)key, key_size) % ht_size;
  for (int step = 0; step < 10; step++) {
    int pos = ht[slot];
    if (pos < 0) return -1;
    if (tab[pos] == *key) return pos;
    slot = (slot + 1) % ht_size;
  }
  return -1;
}

#endif /* SVM_PORT_RUNTIME_H_ */
