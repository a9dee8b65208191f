// Clean-room stand-in for Cow's Variant: only the NamedValues type that the
// reference's Mara.hpp names.  TEST INFRASTRUCTURE.
#pragma once

#include <map>
#include <string>

class Variant
{
public:
    using NamedValues = std::map<std::string, Variant>;
};
