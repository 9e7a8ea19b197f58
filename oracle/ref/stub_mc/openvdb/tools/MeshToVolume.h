#pragma once
#include <openvdb/openvdb.h>
