// CadR/Exceptions.h - the exception classes of CadR's C++ interface
// (reference: src/CadR/Exceptions.h:13-40, same names and meaning).  They
// are thrown by the C++ facade only; the C ABI below it returns status codes.
#pragma once

#include <stdexcept>
#include <string>

#include "../cadr_cuda.h"

namespace CadR {

class Error {
public:
    virtual ~Error() = default;
    virtual const char* what() const noexcept = 0;
};

class LogicError : public Error, public std::logic_error {
public:
    const char* what() const noexcept override { return std::logic_error::what(); }
    explicit LogicError(const std::string& w) : std::logic_error(w) {}
};

class OutOfResources : public Error, public std::runtime_error {
public:
    const char* what() const noexcept override { return std::runtime_error::what(); }
    explicit OutOfResources(const std::string& w) : std::runtime_error(w) {}
};

class Timeout : public Error, public std::runtime_error {
public:
    const char* what() const noexcept override { return std::runtime_error::what(); }
    explicit Timeout(const std::string& w) : std::runtime_error(w) {}
};

// Maps a cadr_status to the exception the reference would throw.
inline void check(cadr_status s, const char* what)
{
    if (s == CADR_OK) return;
    std::string m = std::string(what) + ": " + cadr_last_error();
    if (s == CADR_ERR_OUT_OF_MEMORY || s == CADR_ERR_REJECTED) throw OutOfResources(m);
    if (s == CADR_ERR_TIMEOUT) throw Timeout(m);
    throw LogicError(m);
}

}  // namespace CadR
