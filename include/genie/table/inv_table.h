// genie/table/inv_table.h -- a resident inverted index (the reference's
// inv_table after cpy_data_to_gpu, src/genie/table/inv_table.h).  It owns a
// genie_index handle of the C ABI; ids live on the device.
#ifndef GENIE_TABLE_INV_TABLE_H_
#define GENIE_TABLE_INV_TABLE_H_

#include <cstdint>
#include <string>
#include <vector>

struct genie_index;

namespace genie {
namespace table {

class inv_table {
  public:
    // Row-major n_objects x n_dims values.
    inv_table(const int32_t *values, int64_t n_objects, int32_t n_dims);
    explicit inv_table(genie_index *adopt);
    ~inv_table();
    inv_table(const inv_table &) = delete;
    inv_table &operator=(const inv_table &) = delete;

    int i_size() const;       // objects
    int m_size() const;       // dims
    int64_t inv_size() const; // posting entries
    // The device posting array (ids ordered by (dim, value, id)), as inv().
    std::vector<int> inv() const;
    void save(const std::string &filename) const;
    static inv_table *load(const std::string &filename);
    genie_index *handle() const { return ix_; }

  private:
    genie_index *ix_ = nullptr;
};

}  // namespace table
}  // namespace genie

#endif
