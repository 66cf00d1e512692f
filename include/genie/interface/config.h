// genie/interface/config.h -- search configuration builder
// (reference src/genie/interface/config.h:20-95).
#ifndef GENIE_INTERFACE_CONFIG_H_
#define GENIE_INTERFACE_CONFIG_H_

#include <cstdint>
#include <string>

namespace genie {

class Config {
  public:
    uint32_t GetK() const;
    uint32_t GetQueryRange() const;
    uint32_t GetNumOfQueries() const;
    bool GetSaveToGpu() const;
    uint8_t GetGpuId() const;
    Config &SetK(const uint32_t k);
    Config &SetQueryRange(const uint32_t query_range);
    Config &SetNumOfQueries(const uint32_t num_of_queries);
    Config &SetSaveToGpu(const bool save_to_gpu);
    Config &SetGpuId(const uint8_t gpu_id);
    // Reads "key value" lines (k, query_range, num_of_queries, save_to_gpu, gpu_id).
    Config &LoadFromFile(const std::string &filename);
    bool IsKSet() const;
    bool IsQueryRangeSet() const;
    bool IsNumOfQueriesSet() const;
    // Throws InvalidConfigurationException when K or the number of queries is unset.
    void Validate() const;
    void DisplayConfiguration();

  private:
    uint32_t k_ = 0;
    uint32_t query_range_ = 0;
    uint32_t num_of_queries_ = 0;
    bool save_to_gpu_ = false;
    uint8_t gpu_id_ = 0;
    bool k_initialized_ = false;
    bool query_range_initialized_ = false;
    bool num_of_queries_initialized_ = false;
};

}  // namespace genie

#endif
