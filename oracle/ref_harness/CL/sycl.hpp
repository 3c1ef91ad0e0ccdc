/* Empty stand-in for the SYCL header: the reference's CPU BFS program includes
 * <CL/sycl.hpp> (BFS/cpu_BFS/main.cpp:3) and says `using namespace sycl`
 * (Graph.h:4) but uses nothing from it. */
#pragma once
namespace sycl {}
