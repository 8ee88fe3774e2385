// Error hierarchy mirroring icrar::exception (LA/exception/exception.h:35-92):
// every error carries the throwing file and line.
#pragma once

#include <stdexcept>
#include <string>

namespace icrar {

class exception : public std::exception {
 public:
  exception(const std::string& msg, const std::string& file, int line)
      : m_message(file + ":" + std::to_string(line) + " " + msg) {}
  const char* what() const noexcept override { return m_message.c_str(); }

 private:
  std::string m_message;
};

class invalid_argument_exception : public exception {
 public:
  invalid_argument_exception(const std::string& msg, const std::string& arg, const std::string& file, int line)
      : exception(arg + " invalid argument exception: " + msg, file, line) {}
};

class file_exception : public exception {
 public:
  file_exception(const std::string& filename, const std::string& msg, const std::string& file, int line)
      : exception(filename + " file exception: " + msg, file, line) {}
};

class not_implemented_exception : public exception {
 public:
  not_implemented_exception(const std::string& file, int line) : exception("not implemented", file, line) {}
};

}  // namespace icrar
