// Stand-in for Phase's src/System/Exception.h (Exception.h:7-18).
#pragma once
#include <exception>
#include <string>
class Exception : public std::exception {
 public:
  Exception(const std::string &cls, const std::string &method,
            const std::string &what)
      : message_(cls + "::" + method + " -> " + what) {}
  const char *what() const noexcept override { return message_.c_str(); }
 private:
  std::string message_;
};
