/* intrin.h -- compatibility header for building the reference's grid-key
 * code with g++ through its MSVC branch (test infrastructure only).
 *
 * The reference's UIntKey96::matching_leading_bits / UIntKey64::
 * matching_leading_bits (src/UIntKey96.h:240-265, src/UIntKey64.h:217-240)
 * are complete only in their _MSC_VER branch, which includes <intrin.h> and
 * calls _BitScanReverse; the __GNUC__ branch is an unfinished stub. This
 * header supplies that one intrinsic with its documented meaning: store the
 * bit position of the most significant set bit of `mask` in *index and
 * return nonzero, or return 0 (leaving *index alone) when mask is 0.
 *
 * MSVC's unsigned long is 32 bits; the reference passes the address of a
 * uint32_t, so exactly 4 bytes are stored.
 */
#pragma once
#include <stdint.h>

static inline unsigned char _BitScanReverse(unsigned long* index, unsigned long mask)
{
	const uint32_t m = (uint32_t)mask;
	if (m == 0u) return 0;
	uint32_t pos = 31u;
	while (!(m >> pos)) --pos;
	*(uint32_t*)index = pos;
	return 1;
}
