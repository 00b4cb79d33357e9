// XORWOW random number engine over a structure-of-arrays state, and the
// sampling distributions the EM stepping loop draws from.
//
// Engine semantics follow src/celeritas/random/XorwowRngEngine.hh:191-245
// (Marsaglia xorwow with a Weyl sequence); canonical reals follow
// src/celeritas/random/detail/GenerateCanonical32.hh:63-96 (FP64 uses two
// 32-bit draws, FP32 one). Distributions follow
// src/celeritas/random/distribution/*.hh.
//
// The state lives in six separate 32-bit arrays so that a warp loads each
// word with one coalesced 128-byte transaction; the engine caches the words
// in registers and writes them back once when it goes out of scope.
#pragma once

#include "Types.hh"

namespace gbx
{
//! Per-slot XORWOW state arrays (SoA)
struct RngStateRef
{
    std::uint32_t* s[5];
    std::uint32_t* weyl;
};

//! SplitMix64 (Steele, Lea and Flood 2014; Vigna's constants): a 64-bit
//! counter-based generator used only to expand a seed into XORWOW states
struct SplitMix64
{
    std::uint64_t state;

    GBX_FORCEINLINE std::uint64_t operator()()
    {
        std::uint64_t z = (state += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
};

//! Seed one slot's XORWOW state from a 64-bit key: three SplitMix64 outputs
//! fill the five xor words and the Weyl word, as the reference's
//! XorwowRngEngine initializer does (without its subsequence skip-ahead)
GBX_FORCEINLINE void seed_xorwow(RngStateRef const& ref, size_type slot, std::uint64_t key)
{
    SplitMix64 sm{key};
    std::uint64_t v = sm();
    ref.s[0][slot] = static_cast<std::uint32_t>(v);
    ref.s[1][slot] = static_cast<std::uint32_t>(v >> 32);
    v = sm();
    ref.s[2][slot] = static_cast<std::uint32_t>(v);
    ref.s[3][slot] = static_cast<std::uint32_t>(v >> 32);
    v = sm();
    ref.s[4][slot] = static_cast<std::uint32_t>(v);
    ref.weyl[slot] = static_cast<std::uint32_t>(v >> 32);
    if ((ref.s[0][slot] | ref.s[1][slot] | ref.s[2][slot] | ref.s[3][slot]
         | ref.s[4][slot])
        == 0)
    {
        // XORWOW's xor words must not all vanish
        ref.s[0][slot] = 1;
    }
}

//! XORWOW's F2-linear state transition (the xor words only; the Weyl word
//! is advanced separately)
GBX_FORCEINLINE void xorwow_transition(std::uint32_t* x)
{
    std::uint32_t const t = x[0] ^ (x[0] >> 2u);
    x[0] = x[1];
    x[1] = x[2];
    x[2] = x[3];
    x[3] = x[4];
    x[4] = (x[4] ^ (x[4] << 4u)) ^ (t ^ (t << 1u));
}

//! Apply T^d to the xor words given g(z) = z^d mod p(z), p the
//! characteristic polynomial of the transition T: since p(T) = 0,
//! T^d = g(T) = sum_m g_m T^m. 'poly' holds the 160 coefficients g_m, bit m
//! of the 160-bit integer whose 32-bit words are poly[0] (low) .. poly[4].
GBX_FORCEINLINE void xorwow_apply_poly(std::uint32_t const* poly, std::uint32_t* x)
{
    std::uint32_t acc[5] = {0, 0, 0, 0, 0};
    for (int w = 0; w < 5; ++w)
    {
        std::uint32_t const word = poly[w];
        for (int b = 0; b < 32; ++b)
        {
            if ((word >> b) & 1u)
            {
                for (int k = 0; k < 5; ++k)
                    acc[k] ^= x[k];
            }
            xorwow_transition(x);
        }
    }
    for (int k = 0; k < 5; ++k)
        x[k] = acc[k];
}

//! Advance the xor words by 'count' units, where table[i] is the jump
//! polynomial of 4^i units (one unit: one step, or one subsequence of 2^67
//! steps): base-4 digits of the count, smallest jump first
//! (XorwowRngEngine::jump, src/celeritas/random/XorwowRngEngine.hh:247-265)
GBX_FORCEINLINE void
xorwow_jump(std::uint32_t const* table, unsigned long long count, std::uint32_t* x)
{
    for (int i = 0; count > 0; ++i, count >>= 2)
    {
        for (unsigned int n = static_cast<unsigned int>(count & 3u); n > 0; --n)
            xorwow_apply_poly(table + 5 * i, x);
    }
}

//! Reseed one slot for an event as the reference's reseed_rng does
//! (src/celeritas/random/RngReseed.cc:27-47): state from SplitMix64 of the
//! seed (XorwowRngEngine::operator=(Initializer_t), XorwowRngEngine.hh:164-185),
//! then 'event * num_slots + slot' subsequences ahead; the Weyl word is
//! unchanged by whole subsequences (its period 2^32 divides 2^67).
GBX_FORCEINLINE void reseed_xorwow_slot(RngStateRef const& ref,
                                        std::uint32_t const* subsequence_table,
                                        unsigned int seed,
                                        unsigned long long subsequence,
                                        size_type slot)
{
    SplitMix64 sm{seed};
    std::uint32_t x[5];
    std::uint64_t v = sm();
    x[0] = static_cast<std::uint32_t>(v);
    x[1] = static_cast<std::uint32_t>(v >> 32);
    v = sm();
    x[2] = static_cast<std::uint32_t>(v);
    x[3] = static_cast<std::uint32_t>(v >> 32);
    v = sm();
    x[4] = static_cast<std::uint32_t>(v);
    ref.weyl[slot] = static_cast<std::uint32_t>(v >> 32);
    xorwow_jump(subsequence_table, subsequence, x);
    for (int k = 0; k < 5; ++k)
        ref.s[k][slot] = x[k];
}

class XorwowEngine
{
  public:
    using result_type = std::uint32_t;

    GBX_FORCEINLINE XorwowEngine(RngStateRef const& ref, size_type slot)
        : ref_(ref), slot_(slot)
    {
        for (int i = 0; i < 5; ++i)
            s_[i] = ref.s[i][slot];
        w_ = ref.weyl[slot];
    }
    GBX_FORCEINLINE ~XorwowEngine() { this->store(); }

    XorwowEngine(XorwowEngine const&) = delete;
    XorwowEngine& operator=(XorwowEngine const&) = delete;

    GBX_FORCEINLINE result_type operator()()
    {
        std::uint32_t const t = (s_[0] ^ (s_[0] >> 2u));
        s_[0] = s_[1];
        s_[1] = s_[2];
        s_[2] = s_[3];
        s_[3] = s_[4];
        s_[4] = (s_[4] ^ (s_[4] << 4u)) ^ (t ^ (t << 1u));
        w_ += 362437u;
        return w_ + s_[4];
    }

    GBX_FORCEINLINE void store() const
    {
        for (int i = 0; i < 5; ++i)
            ref_.s[i][slot_] = s_[i];
        ref_.weyl[slot_] = w_;
    }

  private:
    RngStateRef ref_;
    size_type slot_;
    std::uint32_t s_[5];
    std::uint32_t w_;
};

//---------------------------------------------------------------------------//
// Canonical reals in [0, 1)
template<class T>
struct GenerateCanonical;

template<>
struct GenerateCanonical<double>
{
    template<class G>
    GBX_FORCEINLINE double operator()(G& rng) const
    {
        std::uint32_t upper = rng();
        std::uint32_t lower = rng();
        constexpr double norm = 1.1102230246251565e-16;  // 2^-53
        return norm
               * static_cast<double>(
                   (static_cast<std::uint64_t>(upper) << (53u - 32u))
                   ^ static_cast<std::uint64_t>(lower));
    }
};

template<>
struct GenerateCanonical<float>
{
    template<class G>
    GBX_FORCEINLINE float operator()(G& rng) const
    {
        constexpr float norm = 2.32830643654e-10f;  // 2^-32
        return norm * rng();
    }
};

template<class T = real_type, class G>
GBX_FORCEINLINE T generate_canonical(G& rng)
{
    return GenerateCanonical<T>{}(rng);
}

//---------------------------------------------------------------------------//
// Distributions
//---------------------------------------------------------------------------//
//! Uniform in [a, b): fma(b - a, u, a)
template<class T = real_type>
struct UniformRealDistribution
{
    T a;
    T delta;
    GBX_FORCEINLINE UniformRealDistribution(T lo, T hi) : a(lo), delta(hi - lo)
    {
    }
    template<class G>
    GBX_FORCEINLINE T operator()(G& rng) const
    {
        return gbx_fma(delta, generate_canonical<T>(rng), a);
    }
};

//! Exponential with unit mean: log(u) * -1
template<class T = real_type, class G>
GBX_FORCEINLINE T sample_exponential(G& rng)
{
    T const neg_inv_lambda = T{-1} / T{1};
    return libm::log(generate_canonical<T>(rng)) * neg_inv_lambda;
}

//! Bernoulli trial: u < p
template<class T = real_type, class G>
GBX_FORCEINLINE bool sample_bernoulli(T p_true, G& rng)
{
    return generate_canonical<T>(rng) < p_true;
}

//! Bernoulli trial with unnormalized weights for true and false
GBX_FORCEINLINE real_type bernoulli_p(real_type scaled_true,
                                      real_type scaled_false)
{
    return scaled_true / (scaled_true + scaled_false);
}

//! Reciprocal (log-uniform) distribution on [a, b]
template<class T = real_type>
struct ReciprocalDistribution
{
    T a;
    T logratio;
    GBX_FORCEINLINE ReciprocalDistribution(T lo, T hi)
        : a(lo), logratio(libm::log((1 / lo) * hi))
    {
    }
    template<class G>
    GBX_FORCEINLINE T operator()(G& rng) const
    {
        return a * libm::exp(logratio * generate_canonical<T>(rng));
    }
};

//! Rejection test: true if the sample f should be rejected against fmax
template<class T = real_type, class G>
GBX_FORCEINLINE bool reject_sample(T f, T fmax, G& rng)
{
    return f < fmax * generate_canonical<T>(rng);
}

//! Box-Muller normal distribution caching the spare value
template<class T = real_type>
class NormalDistribution
{
  public:
    GBX_FORCEINLINE NormalDistribution(T mean, T stddev)
        : mean_(mean), stddev_(stddev)
    {
    }
    template<class G>
    GBX_FORCEINLINE T operator()(G& rng)
    {
        if (has_spare_)
        {
            has_spare_ = false;
            return gbx_fma(spare_, stddev_, mean_);
        }
        constexpr T twopi = static_cast<T>(2 * constants::pi);
        T theta = twopi * generate_canonical<T>(rng);
        T r = std::sqrt(-2 * libm::log(generate_canonical<T>(rng)));
        spare_ = r * libm::cos(theta);
        has_spare_ = true;
        return gbx_fma(r * libm::sin(theta), stddev_, mean_);
    }

  private:
    T mean_;
    T stddev_;
    T spare_{};
    bool has_spare_{false};
};

//! Poisson: direct product method below lambda=16, else rounded normal
template<class T = real_type, class G>
GBX_FORCEINLINE unsigned int sample_poisson(T lambda, G& rng)
{
    if (lambda <= 16)
    {
        int k = 0;
        T p = libm::exp(lambda);
        do
        {
            ++k;
            p *= generate_canonical<T>(rng);
        } while (p > 1);
        return static_cast<unsigned int>(k - 1);
    }
    NormalDistribution<T> sample_normal(lambda, std::sqrt(lambda));
    return static_cast<unsigned int>(sample_normal(rng) + T(0.5));
}

//! Isotropic unit vector
template<class T = real_type, class G>
GBX_FORCEINLINE Vec3<T> sample_isotropic(G& rng)
{
    T const costheta = UniformRealDistribution<T>(-1, 1)(rng);
    T const phi = UniformRealDistribution<T>(0, 2 * constants::pi)(rng);
    return from_spherical(costheta, phi);
}

//! Rotate a polar cosine with uniform azimuth about a direction
template<class T = real_type, class G>
GBX_FORCEINLINE Vec3<T>
sample_exiting_direction(T costheta, Vec3<T> const& dir, G& rng)
{
    T phi = UniformRealDistribution<T>(0, 2 * constants::pi)(rng);
    return rotate(from_spherical(costheta, phi), dir);
}

}  // namespace gbx
