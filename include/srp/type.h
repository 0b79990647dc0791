/* srp-gb300 public API: scalar type tags.
 *
 * Drop-in replacement for include/srp/type.h of kitrofimov/srp (type.h:17-29).
 * The enumerator order is part of the ABI and must not change. */
#pragma once

#include <stddef.h>
#include <stdint.h>

/** Scalar types understood by the library (index buffers and varyings). */
typedef enum SRPType
{
	SRP_FLOAT = 0,
	SRP_DOUBLE,
	SRP_INT8,
	SRP_INT16,
	SRP_INT32,
	SRP_INT64,
	SRP_UINT8,
	SRP_UINT16,
	SRP_UINT32,
	SRP_UINT64
} SRPType;
