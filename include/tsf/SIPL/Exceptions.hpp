// SIPL/Exceptions.hpp -- the exception types the reference's API throws
// (SIPL::SIPLException, SIPL::IOException; the SIPL submodule is not part of
// the reference tree).  Same names and catch hierarchy so that code written
// against the reference compiles and catches unchanged.
#ifndef TSF_SIPL_EXCEPTIONS_HPP
#define TSF_SIPL_EXCEPTIONS_HPP

#include <stdexcept>
#include <string>

namespace SIPL {

class SIPLException : public std::runtime_error {
public:
    SIPLException() : std::runtime_error("SIPL exception") {}
    explicit SIPLException(const char *message) : std::runtime_error(message) {}
    explicit SIPLException(const std::string &message) : std::runtime_error(message) {}
    SIPLException(const char *message, int line, const char *file)
        : std::runtime_error(std::string(message) + " (" + file + ":" + std::to_string(line) + ")"),
          line_(line), file_(file) {}
    int getLine() const { return line_; }
    const char *getFile() const { return file_; }

private:
    int line_ = -1;
    const char *file_ = "";
};

class IOException : public SIPLException {
public:
    IOException() : SIPLException("IO exception") {}
    explicit IOException(const char *filename) : SIPLException(std::string("Could not open file ") + filename),
                                                 filename_(filename) {}
    IOException(const char *filename, int line, const char *file)
        : SIPLException((std::string("Could not open file ") + filename).c_str(), line, file), filename_(filename) {}
    const std::string &getFilename() const { return filename_; }

private:
    std::string filename_;
};

}  // namespace SIPL
#endif
