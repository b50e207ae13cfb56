/* Reference test fixtures restated for the oracle's own pinning tests. */
#ifndef RD_ORACLE_FIXTURES_H
#define RD_ORACLE_FIXTURES_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
void ro_fixture_amaze_golden(int width, int height, float* out);
void ro_fixture_amaze_probe(float* out);
uint64_t ro_fnv1a_f32(const float* values, size_t count);
#ifdef __cplusplus
}
#endif
#endif
