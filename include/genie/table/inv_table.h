// genie/table/inv_table.h -- a resident inverted index (the reference's
// inv_table after cpy_data_to_gpu, src/genie/table/inv_table.h).  It owns a
// genie_index handle of the C ABI; ids live on the device.
//
// A default-constructed table is empty until one of the legacy loaders
// (genie::original::load_table*, preprocess_for_knn_csv) fills it, as the
// reference's `new inv_table[n]` + load_table pattern does.
#ifndef GENIE_TABLE_INV_TABLE_H_
#define GENIE_TABLE_INV_TABLE_H_

#include <cstdint>
#include <string>
#include <vector>

struct genie_index;

typedef unsigned long long u64;

namespace genie {
namespace table {

class inv_table {
  public:
    inv_table();
    // Row-major n_objects x n_dims values.
    inv_table(const int32_t *values, int64_t n_objects, int32_t n_dims);
    explicit inv_table(genie_index *adopt);
    virtual ~inv_table();
    inv_table(const inv_table &) = delete;
    inv_table &operator=(const inv_table &) = delete;

    int i_size() const;       // objects (for a subsequence table: rows << shift bits)
    int m_size() const;       // dims
    int64_t inv_size() const; // posting entries
    bool empty() const { return ix_ == nullptr; }
    // Host copy of the device posting array (ids ordered by (dim, value,
    // id)), refreshed by every call; the pointer stays valid while the table
    // lives (inv_table::inv, inv_table.cu:248).
    std::vector<int> *inv();
    void save(const std::string &filename) const;
    static inv_table *load(const std::string &filename);
    genie_index *handle() const { return ix_; }
    // Replace the index held (the legacy loaders); the old one is released.
    void adopt(genie_index *ix);

    // Position of this table among the tables of a multiload split.
    void set_table_index(int attr_index) { table_index = attr_index; }
    int get_table_index() const { return table_index; }
    void set_total_num_of_table(int num) { total_num_of_table = num; }
    int get_total_num_of_table() const { return total_num_of_table; }

    // Subsequence tables: a posting id is rowID << bits | offset in the row.
    unsigned int _shift_bits_subsequence() const { return shift_bits_subsequence; }
    void set_shift_bits_subsequence(unsigned int bits) { shift_bits_subsequence = bits; }

    // Sequence (gram) tables: value range of the source sequences and gram length.
    void set_min_value_sequence(int v) { min_value_sequence = v; }
    int get_min_value_sequence() const { return min_value_sequence; }
    void set_max_value_sequence(int v) { max_value_sequence = v; }
    int get_max_value_sequence() const { return max_value_sequence; }
    void set_gram_length_sequence(int g) { gram_length_sequence = g; }
    int get_gram_length_sequence() const { return gram_length_sequence; }
    // Gram values of a sequence table -> the table's value ids (one dim).
    const std::vector<std::pair<int, int> > &distinct_sequence() const { return distinct_; }
    void set_distinct_sequence(std::vector<std::pair<int, int> > d) { distinct_ = std::move(d); }

    // The device posting array (read only), as the reference's d_inv_p.
    int *d_inv_p = nullptr;
    bool is_stored_in_gpu = true;
    int shift_bits_sequence = 0;

  private:
    genie_index *ix_ = nullptr;
    std::vector<int> inv_host_;
    int table_index = 0;
    int total_num_of_table = 1;
    unsigned int shift_bits_subsequence = 0;
    int min_value_sequence = 0;
    int max_value_sequence = 0;
    int gram_length_sequence = 0;
    std::vector<std::pair<int, int> > distinct_;   // sorted (gram value, value id)
};

}  // namespace table
}  // namespace genie

#endif
