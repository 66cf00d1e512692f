// genie/exception/exception.h -- the error types of the C++ interface.
// Same names and bases as the reference's (src/genie/exception/exception.h:10-46);
// the shim maps every C-ABI status code to one of them.
#ifndef GENIE_EXCEPTION_EXCEPTION_H_
#define GENIE_EXCEPTION_EXCEPTION_H_

#include <stdexcept>
#include <string>

namespace genie {
namespace exception {

class NotImplementedException : public std::logic_error {
  public:
    NotImplementedException() : std::logic_error("Function is not implemented") {}
};

class InvalidConfigurationException : public std::logic_error {
  public:
    explicit InvalidConfigurationException(const std::string &what) : std::logic_error(what) {}
};

class gpu_bad_alloc : public std::runtime_error {
  public:
    explicit gpu_bad_alloc(const std::string &what) : std::runtime_error(what) {}
};

class gpu_runtime_error : public std::runtime_error {
  public:
    explicit gpu_runtime_error(const std::string &what) : std::runtime_error(what) {}
};

class cpu_bad_alloc : public std::runtime_error {
  public:
    explicit cpu_bad_alloc(const std::string &what) : std::runtime_error(what) {}
};

class cpu_runtime_error : public std::runtime_error {
  public:
    explicit cpu_runtime_error(const std::string &what) : std::runtime_error(what) {}
};

// Throw the exception type of a genie_status code (no-op for GENIE_OK), with
// the library's last error message.
void throw_on_status(int status);

}  // namespace exception
}  // namespace genie

#endif
