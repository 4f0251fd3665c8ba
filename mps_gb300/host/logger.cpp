#include "logger.hpp"

#include <chrono>
#include <ctime>
#include <iostream>

namespace mpslog {
namespace {
std::ofstream g_file;
const char* names[] = {"debug", "info", "warning", "error"};
std::string stamp() {
    std::time_t t = std::time(nullptr);
    char buf[32];
    std::strftime(buf, sizeof buf, "%Y-%m-%d %H:%M:%S", std::localtime(&t));
    return buf;
}
}  // namespace

void open_file(const std::string& path) { g_file.open(path, std::ios::trunc); }
void close_file() {
    if (g_file.is_open()) g_file.close();
}
void log(Level lv, const std::string& msg) {
    std::string line = "[" + stamp() + "] [" + names[lv] + "] " + msg;
    if (lv >= Info) std::cout << line << std::endl;
    if (g_file.is_open()) {
        g_file << line << '\n';
        if (lv >= Error) g_file.flush();
    }
}
}  // namespace mpslog
