/* srp-gb300 public API: error and warning reporting.
 *
 * Drop-in replacement for include/srp/message_callback.h of kitrofimov/srp
 * (message_callback.h:14-45). The library never returns error codes from the
 * srp* API; it reports through this callback and then returns. CUDA errors are
 * reported the same way as SRP_MESSAGE_ERROR / SRP_MESSAGE_SEVERITY_HIGH. */
#pragma once

/** Kind of a message. */
typedef enum SRPMessageType
{
	SRP_MESSAGE_ERROR,
	SRP_MESSAGE_WARNING
} SRPMessageType;

/** Severity of a message. */
typedef enum SRPMessageSeverity
{
	SRP_MESSAGE_SEVERITY_LOW,
	SRP_MESSAGE_SEVERITY_MODERATE,
	SRP_MESSAGE_SEVERITY_HIGH
} SRPMessageSeverity;

/** User hook: receives the message kind, severity, the name of the library
 *  function that raised it, the formatted text and the user pointer. */
typedef void (*SRPMessageCallbackFunc)(
	SRPMessageType type, SRPMessageSeverity severity, const char* sourceFunction,
	const char* message, void* userParameter
);

/** Callback plus the opaque pointer handed back to it. */
typedef struct SRPMessageCallback
{
	SRPMessageCallbackFunc func;
	void* userParameter;
} SRPMessageCallback;
