// genie/utility/Logger.h -- leveled console logging of the legacy interface
// (reference src/genie/utility/Logger.h:41-148).  Messages at or below the
// set level go to stderr; nothing is written to files.
#ifndef GENIE_UTILITY_LOGGER_H_
#define GENIE_UTILITY_LOGGER_H_

namespace genie {
namespace utility {

class Logger {
  public:
    static const int NONE = 0;
    static const int ALERT = 1;
    static const int INFO = 2;
    static const int VERBOSE = 3;
    static const int DEBUG = 4;

    static void exit(void);
    static int log(int level, const char *fmt, ...);
    static void set_level(int level);
    static int get_level();
    static void set_logfile_name(const char *name);
    static const char *get_logfile_name();
};

}  // namespace utility
}  // namespace genie

#endif
