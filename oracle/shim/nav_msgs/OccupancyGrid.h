// TEST INFRASTRUCTURE ONLY: stand-in header, see ros_stub.hpp.
#pragma once
#include "../ros_stub.hpp"
