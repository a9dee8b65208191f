// Clean-room stand-in for Cow's Logger: a sink that discards everything.
// TEST INFRASTRUCTURE (lets the reference's Mara.hpp compile).
#pragma once

#include <ostream>
#include <string>

class Logger
{
public:
    Logger() : null (nullptr) {}
    std::ostream& log (std::string = "") { return null; }
private:
    std::ostream null;
};
