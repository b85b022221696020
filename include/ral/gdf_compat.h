/*
 * gdf_compat.h — the column, scalar and operator types that the BlazingSQL RAL
 * expression path exchanges with its callers.
 *
 * The reference builds against cudf's C headers (cudf.h, cudf/binaryop.hpp),
 * which are not part of the reference tree.  This header restates the field
 * and enumerator NAMES the reference uses so that a caller of
 * perform_operation / evaluate_expression / process_filter can hand the same
 * structures to this library:
 *   - gdf_column: data buffer + LSB-first validity bitmask (bit i of byte i/8),
 *     used throughout src/Interpreter/interpreter_ops.cuh:1049-1070 and
 *     src/ColumnManipulation.cu:26-68.
 *   - gdf_scalar {data, dtype, is_valid}: src/CalciteExpressionParsing.cpp:337-417.
 *   - gdf_unary_operator: the reference's own enum, same order and therefore
 *     the same numeric values (src/gdf_wrapper/gdf_types.cuh:7-31).
 *   - gdf_dtype / gdf_binary_operator: cudf enums; the numeric values below
 *     follow cudf 0.7/0.8 ordering but are this library's own (cudf's headers
 *     are not available to check against).
 *   - column_index_type, SCALAR_INDEX, SCALAR_NULL_INDEX:
 *     src/Interpreter/interpreter_cpp.h:20-22.
 *
 * Plain C, usable from C, C++, cgo, JNI or ctypes.
 */
#ifndef RAL_GDF_COMPAT_H_
#define RAL_GDF_COMPAT_H_

#include <stdint.h>
#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Row count / index type of that cudf era (32-bit). */
typedef int32_t gdf_size_type;
typedef int32_t gdf_index_type;
/* One byte of validity bitmask; bit i of the column is (valid[i/8] >> (i%8)) & 1. */
typedef uint8_t gdf_valid_type;

typedef enum {
    GDF_invalid = 0,
    GDF_INT8,
    GDF_INT16,
    GDF_INT32,
    GDF_INT64,
    GDF_FLOAT32,
    GDF_FLOAT64,
    GDF_BOOL8,
    GDF_DATE32,     /* days since the UNIX epoch, int32 */
    GDF_DATE64,     /* milliseconds since the UNIX epoch, int64 */
    GDF_TIMESTAMP,  /* int64, unit in dtype_info */
    GDF_CATEGORY,
    GDF_STRING,
    GDF_STRING_CATEGORY,
    N_GDF_TYPES
} gdf_dtype;

typedef enum {
    TIME_UNIT_NONE = 0,
    TIME_UNIT_s,
    TIME_UNIT_ms,
    TIME_UNIT_us,
    TIME_UNIT_ns
} gdf_time_unit;

typedef struct {
    gdf_time_unit time_unit;
    void *category;
} gdf_dtype_extra_info;

typedef struct gdf_column_ {
    void *data;
    gdf_valid_type *valid;     /* may be NULL: every row valid */
    gdf_size_type size;
    gdf_dtype dtype;
    gdf_size_type null_count;
    gdf_dtype_extra_info dtype_info;
    char *col_name;
} gdf_column;

typedef union {
    int8_t si08;
    int16_t si16;
    int32_t si32;
    int64_t si64;
    uint8_t ui08;
    uint16_t ui16;
    uint32_t ui32;
    uint64_t ui64;
    float fp32;
    double fp64;
    int32_t dt32;
    int64_t dt64;
    int64_t tmst;
} gdf_data;

typedef struct {
    gdf_data data;
    gdf_dtype dtype;
    bool is_valid;
} gdf_scalar;

/* Binary operators of the register program (cudf/binaryop.hpp names). */
typedef enum {
    GDF_ADD = 0,
    GDF_SUB,
    GDF_MUL,
    GDF_DIV,
    GDF_TRUE_DIV,
    GDF_FLOOR_DIV,
    GDF_MOD,
    GDF_POW,
    GDF_EQUAL,
    GDF_NOT_EQUAL,
    GDF_LESS,
    GDF_GREATER,
    GDF_LESS_EQUAL,
    GDF_GREATER_EQUAL,
    GDF_BITWISE_AND,
    GDF_BITWISE_OR,
    GDF_BITWISE_XOR,
    GDF_LOGICAL_AND,
    GDF_LOGICAL_OR,
    GDF_COALESCE,
    GDF_GENERIC_BINARY,
    GDF_INVALID_BINARY
} gdf_binary_operator;

/* Unary operators: identical order to src/gdf_wrapper/gdf_types.cuh:7-31. */
typedef enum {
    BLZ_FLOOR = 0,
    BLZ_CEIL,
    BLZ_SIN,
    BLZ_COS,
    BLZ_ASIN,
    BLZ_ACOS,
    BLZ_TAN,
    BLZ_COTAN,
    BLZ_ATAN,
    BLZ_ABS,
    BLZ_NOT,
    BLZ_LN,
    BLZ_LOG,
    BLZ_YEAR,
    BLZ_MONTH,
    BLZ_DAY,
    BLZ_HOUR,
    BLZ_MINUTE,
    BLZ_SECOND,
    BLZ_IS_NULL,
    BLZ_IS_NOT_NULL,
    BLZ_INVALID_UNARY
} gdf_unary_operator;

/* Aggregation operators (cudf's gdf_agg_op, the names src/operators/GroupBy.cpp and
 * src/CalciteExpressionParsing.cpp:92-116,483-507 use; cudf is not vendored by the reference, so
 * the values follow cudf's published order of that era). */
typedef enum {
    GDF_SUM = 0,
    GDF_MIN,
    GDF_MAX,
    GDF_AVG,
    GDF_COUNT,
    GDF_COUNT_DISTINCT,
    N_GDF_AGG_OPS
} gdf_agg_op;

/* Register index type and the two negative operand codes of the program. */
typedef short column_index_type;
#define SCALAR_INDEX ((column_index_type)-2)
#define SCALAR_NULL_INDEX ((column_index_type)-3)
#define UNARY_RIGHT_INDEX ((column_index_type)-1)

/* Byte size of a validity mask for n rows, padded to 64 bytes as the
 * reference allocates it (src/Traits/RuntimeTraits.h:63, GDFColumn.cu:163-173).
 * Every valid buffer handed to this library must be at least this large:
 * kernels read and write whole 32-bit words of it. */
static inline size_t gdf_valid_allocation_size(int64_t n) {
    size_t bytes = (size_t)((n + 7) / 8);
    return ((bytes + 63) / 64) * 64;
}

/* Width in bytes of one element of a fixed-width dtype; 0 if not fixed-width. */
static inline int gdf_dtype_size(gdf_dtype t) {
    switch (t) {
    case GDF_INT8: case GDF_BOOL8: return 1;
    case GDF_INT16: return 2;
    case GDF_INT32: case GDF_FLOAT32: case GDF_DATE32:
    case GDF_CATEGORY: case GDF_STRING_CATEGORY: return 4;
    case GDF_INT64: case GDF_FLOAT64: case GDF_DATE64: case GDF_TIMESTAMP: return 8;
    default: return 0;
    }
}

#ifdef __cplusplus
}
#endif

#endif /* RAL_GDF_COMPAT_H_ */
