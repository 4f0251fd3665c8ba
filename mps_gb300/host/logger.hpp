// Console + file logger with the reference's line format
// "[%Y-%m-%d %H:%M:%S] [level] message" (src/simulation.cpp:79-100):
// info and above to the console, debug and above to the file.
#pragma once
#include <fstream>
#include <string>

namespace mpslog {
enum Level { Debug = 0, Info = 1, Warn = 2, Error = 3 };
void open_file(const std::string& path);
void close_file();
void log(Level lv, const std::string& msg);
inline void debug(const std::string& m) { log(Debug, m); }
inline void info(const std::string& m) { log(Info, m); }
inline void error(const std::string& m) { log(Error, m); }
}  // namespace mpslog
