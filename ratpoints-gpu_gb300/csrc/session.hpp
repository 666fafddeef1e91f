// Definition of the opaque rpg_session handle of the C ABI: a sieve with its
// per-curve tables resident on one device, plus the events that time it.
#pragma once

#include <cuda_runtime.h>

#include <memory>

#include "sieve.hpp"

struct rpg_session {
    std::unique_ptr<rpg::Sieve> sieve;
    cudaEvent_t begin = nullptr, end = nullptr;
    ~rpg_session() {
        if (begin) cudaEventDestroy(begin);
        if (end) cudaEventDestroy(end);
    }
};
