/*
 * gpr_common.h -- op codes, op classes and the compiled-program instruction
 * encoding shared by the host library and the kernels.
 *
 * Op codes keep the reference's numbering (enum OPS, main.cu:53) so chain
 * state moves between the reference layout and this library unchanged.
 * Each op's arity, description-length cost (dispatch_length, main.cu:477-526)
 * and node count (dispatch_countnodes, main.cu:553-601) is a property of its
 * class below.
 */
#ifndef GPR_COMMON_H
#define GPR_COMMON_H

#include <stdint.h>

enum gpr_op {
    OP_ONE = 0, OP_CONST, OP_INV, OP_A, OP_B, OP_PLUS, OP_MINUS, OP_RMINUS, OP_CPLUS,
    OP_TIMES, OP_CTIMES, OP_DIV, OP_RDIV, OP_LOG, OP_EXP, OP_POW, OP_CPOW, OP_RPOW,
    OP_CRPOW, OP_SQRT, OP_SIN, OP_ASIN, OP_COS, OP_ACOS, OP_TAN, OP_ATAN, OP_ABS,
    OP_NREF, /* 27 = NOPS of the reference's default op set */
    /* leaves of multivariate data (no reference counterpart): the input
     * variables x1, x2, x3.  A child beyond the heap is x1, as the
     * reference's x (main.cu:374-385). */
    OP_X1 = OP_NREF, OP_X2, OP_X3,
    OP_NALL
};

/* PROGRAM_CODE, main.cu:55: one character per op, used in samples.txt; the
 * variable leaves x1, x2, x3 print as X, Y, Z. */
#define GPR_PROGRAM_CODE "1CIab+-_#*@/|LE^pVPRSsCcTtAXYZ"

enum gpr_opclass {
    CLS_LEAF0 = 0,   /* ONE, CONST: no children                                  */
    CLS_PASS_A,      /* A: value of the left child                               */
    CLS_PASS_B,      /* B: value of the right child                              */
    CLS_UNARY,       /* f(a): length 1+a, count 1+a                              */
    CLS_CUNARY,      /* f(a, C): length CONST_LENGTH_PRIOR+a+1, count a+1        */
    CLS_BINARY,      /* g(a, b): length 1+a+b, count 1+a+b                       */
    CLS_INVALID
};

#if defined(__CUDACC__)
#define GPR_HDI __host__ __device__ __forceinline__
#else
#define GPR_HDI static inline
#endif

/* The class of op o: a 4-bit field per op, eight ops to a 32-bit word, so
 * the lookup is a few integer operations with no branch or jump table. */
#define GPR_CLS_AT(op, cls) ((uint32_t)(cls) << (4 * ((op) & 7)))
#define GPR_CLS_WORD(w)                                                                               \
    ((uint32_t)(GPR_CLS_FIELD((w) * 8 + 0) | GPR_CLS_FIELD((w) * 8 + 1) | GPR_CLS_FIELD((w) * 8 + 2) | \
                GPR_CLS_FIELD((w) * 8 + 3) | GPR_CLS_FIELD((w) * 8 + 4) | GPR_CLS_FIELD((w) * 8 + 5) | \
                GPR_CLS_FIELD((w) * 8 + 6) | GPR_CLS_FIELD((w) * 8 + 7)))
#define GPR_CLS_FIELD(op) GPR_CLS_AT(op, gpr_op_class_slow(op))

#if defined(__CUDACC__)
#define GPR_HDC __host__ __device__ constexpr
#else
#define GPR_HDC static constexpr
#endif

/* The class of op o, written out; only evaluated at compile time, to build
 * the table below. */
GPR_HDC int gpr_op_class_slow(int o) {
    return (o == OP_ONE || o == OP_CONST || o == OP_X1 || o == OP_X2 || o == OP_X3) ? CLS_LEAF0
         : o == OP_A ? CLS_PASS_A
         : o == OP_B ? CLS_PASS_B
         : (o == OP_INV || o == OP_LOG || o == OP_EXP || o == OP_SQRT || o == OP_SIN || o == OP_ASIN ||
            o == OP_COS || o == OP_ACOS || o == OP_TAN || o == OP_ATAN || o == OP_ABS) ? CLS_UNARY
         : (o == OP_CPLUS || o == OP_CTIMES || o == OP_CPOW || o == OP_CRPOW) ? CLS_CUNARY
         : (o == OP_PLUS || o == OP_MINUS || o == OP_RMINUS || o == OP_TIMES || o == OP_DIV || o == OP_RDIV ||
            o == OP_POW || o == OP_RPOW) ? CLS_BINARY
         : CLS_INVALID;
}

GPR_HDI int gpr_op_class(int o) {
    if ((unsigned)o >= 32u) return CLS_INVALID;
    const int w = o >> 3;
    const uint32_t word = w == 0 ? GPR_CLS_WORD(0) : w == 1 ? GPR_CLS_WORD(1) : w == 2 ? GPR_CLS_WORD(2)
                                                                                    : GPR_CLS_WORD(3);
    return (int)((word >> (4 * (o & 7))) & 15u);
}

/* ---- compiled program: a reachable-only postfix form of the heap tree ----
 * One 16-bit word per instruction (gpr_word): bits 0-7 code, bits 8-15 heap
 * node (the constant C[node] an instruction reads).  The evaluator keeps the running
 * value in an accumulator; leaf operands (x1..x3, 1, a constant) are folded into
 * the instruction that consumes them, so the value stack is touched only
 * where both children of a binary node are subtrees. */
typedef uint16_t gpr_word;
enum gpr_icode {
    I_END = 0,
    I_LDX = 1, I_LDC = 2, I_LD1 = 3, I_PUSH = 4, I_LDNAN = 5, I_LDX2 = 6, I_LDX3 = 7,
    U_INV = 8, U_LOG, U_EXP, U_SQRT, U_SIN, U_ASIN, U_COS, U_ACOS, U_TAN, U_ATAN, U_ABS,
    I_BIN0 = 32   /* 32 + bop*16 + accleft*8 + src (3 bits) */
};
enum gpr_bop { BOP_ADD = 0, BOP_SUB = 1, BOP_MUL = 2, BOP_DIV = 3, BOP_POW = 4 };
enum gpr_src { SRC_X = 0, SRC_C = 1, SRC_ONE = 2, SRC_POP = 3, SRC_X2 = 4, SRC_X3 = 5 };

#define GPR_BIN(bop, accleft, src) (I_BIN0 + (bop) * 16 + (accleft) * 8 + (src))
/* fields of a binary instruction code */
#define GPR_BIN_BOP(code) (((code) - I_BIN0) >> 4)
#define GPR_BIN_ACCLEFT(code) (((code) >> 3) & 1u)
#define GPR_BIN_SRC(code) ((code) & 7u)

/* Counters the MH kernel accumulates (gpr_get_stats). */
enum gpr_stat {
    GPR_STAT_EVALS = 0,        /* likelihood evaluations (one per proposal + one per chain) */
    GPR_STAT_EVAL_NODES,       /* sum over evaluations of the program's node count          */
    GPR_STAT_EVAL_POINTS,      /* data points actually evaluated (early exit on invalid)   */
    GPR_STAT_EVAL_NODE_POINTS, /* sum over evaluations of (node count + 4) * points        */
    GPR_STAT_STRUCT_PROPOSED,
    GPR_STAT_STRUCT_ACCEPTED,
    GPR_STAT_CONST_PROPOSED,
    GPR_STAT_CONST_ACCEPTED,
    GPR_NSTATS
};

/* Phases of one chain's block that the instrumented MH kernel times
 * (gpr_debug_phase_profile): clock64 cycles of each warp between phase
 * boundaries, summed over warps.  After the phases, two counts: evaluation
 * passes run, and program instructions interpreted (summed over passes). */
enum gpr_phase {
    GPR_PH_CLAIM = 0,  /* claiming the next chain (group barrier + counter)       */
    GPR_PH_LOAD,       /* chain state in from device memory                        */
    GPR_PH_STEPBAR,    /* step barrier of the free-running / periodic layouts      */
    GPR_PH_STRUCT,     /* structure proposal (main.cu:699-742)                     */
    GPR_PH_CONST,      /* constant proposal (main.cu:743-806)                      */
    GPR_PH_COMPILE,    /* heap tree -> postfix program                             */
    GPR_PH_CAUCHY,     /* Cauchy prior over all constants                          */
    GPR_PH_EPROG,      /* evaluation program (instructions paired with constants)  */
    GPR_PH_BAR1,       /* publishing the program + the first step barrier          */
    GPR_PH_RANK,       /* ranking the CTA's programs by length                     */
    GPR_PH_EVAL,       /* evaluation passes and their reductions                   */
    GPR_PH_BAR2,       /* the second step barrier                                  */
    GPR_PH_COMBINE,    /* combining a chain's pass sums into its likelihood        */
    GPR_PH_ACCEPT,     /* prior, posterior, accept rule, bookkeeping               */
    GPR_PH_STORE,      /* chain state and scores out                               */
    GPR_NPHASES,
    GPR_PH_NPASSES = GPR_NPHASES,   /* count: evaluation passes                    */
    GPR_PH_NINSTR,                  /* count: instructions interpreted             */
    GPR_PH_SLOTS
};

/* Passes (32*K points each) a CTA-balanced evaluation can split a dataset
 * into; beyond it each warp evaluates its own chain. */
#define GPR_MAX_PASSES 64

/* Maximum compiled length for a program of PL heap nodes. */
#define GPR_MAX_INSTR(PL) (2 * (PL) + 4)

#endif /* GPR_COMMON_H */
