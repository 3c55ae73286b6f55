/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Stand-in for the reference's Poisson_noise class (c++/include/poisson_noise.h:10-28)
 * used when the reference's own neuron classes are compiled under oracle/_ref.
 * It keeps the reference's public interface but draws from one counter-based
 * Philox stream per neuron (ugo_noise.h) instead of the rank-wide mt19937, so
 * the reference's code consumes exactly the numbers the oracle and the CUDA
 * kernels consume.  This directory precedes the reference's include directory
 * on the compiler's search path.
 */
#pragma once
#ifndef POISSON_NOISE_H
#define POISSON_NOISE_H

#include <cmath>
#include <iostream>
#include "../ugo_noise.h"

class Poisson_noise
{
public:
    Poisson_noise() { ugo_stream_init(&stream_, 0, 0, 0, 0, 0); }
    void bind(uint64_t seed, uint32_t kind, uint32_t net, uint32_t entity, uint32_t trial)
    {
        ugo_stream_init(&stream_, seed, kind, net, entity, trial);
    }
    void set_seed(unsigned s) { (void)s; }
    double get_spike_time(double lambda) { return -std::log(1 - ugo_u01(ugo_stream_word(&stream_))) / lambda; }
    double random(double G) { return ugo_random_G(G, ugo_stream_word(&stream_)); }
    int sample_index_for_point_distribution() { return ugo_point_index(ugo_stream_word(&stream_)); }
    int sample_integer(int min, int max) { return min + (int)(ugo_stream_word(&stream_) % (uint32_t)(max - min + 1)); }
    void set_normal_distribution(double mu, double sigma) { (void)mu; (void)sigma; }
    double normal_distribution() { return 0.0; }

private:
    ugo_stream stream_;
};

#endif
