/*
 * Minimal stand-in for the OCaml runtime headers, written for this project so
 * that the reference POY C sources (algn.c and the files it pulls in) compile
 * as a plain C library with no OCaml toolchain.
 *
 * This is test infrastructure for the oracle only. Values are tagged integers
 * (OCaml's 2n+1 encoding), custom blocks are a header word followed by the
 * payload, and failwith() jumps back to the harness that called the stub.
 * Root registration (CAMLparam/CAMLlocal) is a no-op: nothing is collected.
 */
#ifndef POY_CAML_SHIM_H
#define POY_CAML_SHIM_H 1

#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

typedef intptr_t value;
typedef uintptr_t header_t;
typedef unsigned long mlsize_t;
typedef unsigned int tag_t;
typedef unsigned long uintnat;
typedef long intnat;

#define Val_long(x) ((value)(((intnat)(x) << 1) + 1))
#define Long_val(v) ((intnat)(v) >> 1)
#define Val_int(x) Val_long(x)
#define Int_val(v) ((int)Long_val(v))
#define Bool_val(v) Int_val(v)
#define Val_bool(x) Val_int((x) != 0)
#define Val_unit Val_int(0)
#define Val_false Val_int(0)
#define Val_true Val_int(1)
#define Val_emptylist Val_int(0)

/* Blocks used by the shim: a word of header, then the fields. */
#define Field(v, i) (((value *)(v))[i])
#define Store_field(b, i, v) (Field((b), (i)) = (v))
#define Wosize_val(v) ((mlsize_t)0)
#define Tag_val(v) ((tag_t)0)
#define Is_block(v) (((v) & 1) == 0)
#define Is_long(v) (((v) & 1) != 0)
#define Double_val(v) (*(double *)(v))
#define String_val(v) ((char *)(v))

/* Custom blocks: [ops pointer][payload ...]. */
struct custom_operations {
    const char *identifier;
    void (*finalize)(value v);
    int (*compare)(value v1, value v2);
    intnat (*hash)(value v);
    void (*serialize)(value v, uintnat *bsize_32, uintnat *bsize_64);
    uintnat (*deserialize)(void *dst);
    int (*compare_ext)(value v1, value v2);
    const void *fixed_length;
};
#define custom_finalize_default NULL
#define custom_compare_default NULL
#define custom_hash_default NULL
#define custom_serialize_default NULL
#define custom_deserialize_default NULL
#define custom_compare_ext_default NULL
#define custom_fixed_length_default NULL
#define Custom_ops_val(v) (*((struct custom_operations **)(v)))
#define Data_custom_val(v) ((void *)(((value *)(v)) + 1))

value caml_alloc_custom(struct custom_operations *ops, uintnat size,
                        mlsize_t mem, mlsize_t max);
#define alloc_custom caml_alloc_custom
void caml_register_custom_operations(struct custom_operations *ops);
#define register_custom_operations caml_register_custom_operations

value caml_alloc(mlsize_t wosize, tag_t tag);
value caml_alloc_tuple(mlsize_t wosize);
value caml_copy_double(double d);
#define alloc caml_alloc
#define alloc_tuple caml_alloc_tuple
#define copy_double caml_copy_double

/* Errors raise through the harness. */
void caml_failwith(const char *msg);
#define failwith caml_failwith
void caml_invalid_argument(const char *msg);
#define invalid_argument caml_invalid_argument

/* Root registration is a no-op in this shim. */
#define CAMLparam0()
#define CAMLparam1(a) (void)(a)
#define CAMLparam2(a, b) (void)(a); (void)(b)
#define CAMLparam3(a, b, c) CAMLparam2(a, b); (void)(c)
#define CAMLparam4(a, b, c, d) CAMLparam3(a, b, c); (void)(d)
#define CAMLparam5(a, b, c, d, e) CAMLparam4(a, b, c, d); (void)(e)
#define CAMLxparam1(a) (void)(a)
#define CAMLxparam2(a, b) (void)(a); (void)(b)
#define CAMLxparam3(a, b, c) CAMLxparam2(a, b); (void)(c)
#define CAMLxparam4(a, b, c, d) CAMLxparam3(a, b, c); (void)(d)
#define CAMLxparam5(a, b, c, d, e) CAMLxparam4(a, b, c, d); (void)(e)
#define CAMLlocal1(a) value a = Val_unit
#define CAMLlocal2(a, b) value a = Val_unit, b = Val_unit
#define CAMLlocal3(a, b, c) value a = Val_unit, b = Val_unit, c = Val_unit
#define CAMLlocal4(a, b, c, d) CAMLlocal2(a, b); CAMLlocal2(c, d)
#define CAMLlocal5(a, b, c, d, e) CAMLlocal3(a, b, c); CAMLlocal2(d, e)
#define CAMLlocalN(x, n) value x[n]
#define CAMLreturn(x) return (x)
#define CAMLreturn0 return
#define CAMLreturnT(t, x) return (x)

/* Serialization hooks (not exercised by the alignment path). */
void caml_serialize_int_1(int i);
void caml_serialize_int_2(int i);
void caml_serialize_int_4(int32_t i);
void caml_serialize_int_8(int64_t i);
void caml_serialize_block_1(void *data, intnat len);
void caml_serialize_block_4(void *data, intnat len);
int caml_deserialize_sint_1(void);
int caml_deserialize_uint_1(void);
int caml_deserialize_sint_2(void);
int caml_deserialize_uint_2(void);
int32_t caml_deserialize_sint_4(void);
uint32_t caml_deserialize_uint_4(void);
int64_t caml_deserialize_sint_8(void);
void caml_deserialize_block_1(void *data, intnat len);
void caml_deserialize_block_4(void *data, intnat len);
#define serialize_int_1 caml_serialize_int_1
#define serialize_int_2 caml_serialize_int_2
#define serialize_int_4 caml_serialize_int_4
#define serialize_int_8 caml_serialize_int_8
#define serialize_block_1 caml_serialize_block_1
#define serialize_block_4 caml_serialize_block_4
#define deserialize_sint_1 caml_deserialize_sint_1
#define deserialize_uint_1 caml_deserialize_uint_1
#define deserialize_sint_2 caml_deserialize_sint_2
#define deserialize_uint_2 caml_deserialize_uint_2
#define deserialize_sint_4 caml_deserialize_sint_4
#define deserialize_uint_4 caml_deserialize_uint_4
#define deserialize_sint_8 caml_deserialize_sint_8
#define deserialize_block_1 caml_deserialize_block_1
#define deserialize_block_4 caml_deserialize_block_4

/* Bigarray views (not exercised by the alignment path). */
struct caml_ba_array {
    void *data;
    intnat num_dims;
    intnat flags;
    void *proxy;
    intnat dim[4];
};
#define Caml_ba_array_val(v) ((struct caml_ba_array *)Data_custom_val(v))
#define Caml_ba_data_val(v) (Caml_ba_array_val(v)->data)
#define Bigarray_val Caml_ba_array_val
#define Data_bigarray_val Caml_ba_data_val
#define CAML_BA_INT32 6
#define CAML_BA_C_LAYOUT 0
#define CAML_BA_FLOAT64 1
#define BIGARRAY_INT32 CAML_BA_INT32
#define BIGARRAY_C_LAYOUT CAML_BA_C_LAYOUT
#define BIGARRAY_FLOAT64 CAML_BA_FLOAT64
value caml_ba_alloc(int flags, int num_dims, void *data, intnat *dim);
value caml_ba_alloc_dims(int flags, int num_dims, void *data, ...);
#define alloc_bigarray caml_ba_alloc
#define alloc_bigarray_dims caml_ba_alloc_dims

#endif /* POY_CAML_SHIM_H */
