/* Minimal declarations of libbrotlienc's public C API (brotli 1.x,
 * <brotli/encode.h>), enough to compile the reference's CPU build against the
 * installed runtime library (libbrotlienc.so.1) when the -dev headers are not
 * installed.  Only the names, enum values and signatures of the public API are
 * given here. */
#ifndef CUBFF_ORACLE_BROTLI_SHIM_ENCODE_H_
#define CUBFF_ORACLE_BROTLI_SHIM_ENCODE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum BrotliEncoderMode {
  BROTLI_MODE_GENERIC = 0,
  BROTLI_MODE_TEXT = 1,
  BROTLI_MODE_FONT = 2
} BrotliEncoderMode;

size_t BrotliEncoderMaxCompressedSize(size_t input_size);

int BrotliEncoderCompress(int quality, int lgwin, BrotliEncoderMode mode,
                          size_t input_size, const uint8_t *input_buffer,
                          size_t *encoded_size, uint8_t *encoded_buffer);

#ifdef __cplusplus
}
#endif

#endif
