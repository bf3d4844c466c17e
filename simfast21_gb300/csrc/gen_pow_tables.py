"""Generate pow_tables.h: fixed-point constants for sd_pow (softdouble.h).

Run:  python gen_pow_tables.py > pow_tables.h
Uses only the standard library (decimal, 60 significant digits)."""
from decimal import Decimal, getcontext

getcontext().prec = 60
LN2 = Decimal(2).ln()


def log2(x):
    return x.ln() / LN2


def rnd(x):
    return int(x.to_integral_value(rounding="ROUND_HALF_EVEN"))


inv = [rnd(Decimal(2) ** 62 / (1 + (Decimal(j) + Decimal("0.5")) / 128)) for j in range(128)]
l2c = [rnd(log2(Decimal(2) ** 62 / Decimal(v)) * Decimal(2) ** 96) for v in inv]
rcp = [0] + [rnd(Decimal(2) ** 124 / k) for k in range(1, 10)]
ifact = []
f = Decimal(1)
for k in range(11):
    if k:
        f *= k
    ifact.append(rnd(Decimal(2) ** 124 / f))
exp2t = [rnd(Decimal(2) ** 124 * (LN2 * Decimal(j) / 128).exp()) for j in range(128)]
inv_ln2 = rnd(Decimal(2) ** 124 / LN2)
log2e_q96 = rnd(Decimal(2) ** 96 / LN2)
ln2 = rnd(Decimal(2) ** 124 * LN2)

M64 = (1 << 64) - 1
out = [
    "// Generated by gen_pow_tables.py -- do not edit.",
    "// Fixed-point constants for sd_pow (softdouble.h).",
    "#pragma once",
    "#include <stdint.h>",
    # the header is compiled once for the host and once for the device; each
    # pass gets its own copy of the tables
    "#if defined(__CUDA_ARCH__)\n#define SD_T static __device__ const\n#else\n#define SD_T static const\n#endif",
]


def arr(name, vals):
    body = ",\n  ".join(", ".join(f"0x{v:016x}ULL" for v in vals[i:i + 4]) for i in range(0, len(vals), 4))
    return f"SD_T uint64_t {name}[{len(vals)}] = {{\n  {body}}};"


out.append(arr("SD_POW_INV", inv))
out.append(arr("SD_POW_L2C_HI", [v >> 64 for v in l2c]))
out.append(arr("SD_POW_L2C_LO", [v & M64 for v in l2c]))
out.append(arr("SD_POW_RCP_HI", [v >> 64 for v in rcp]))
out.append(arr("SD_POW_RCP_LO", [v & M64 for v in rcp]))
out.append(arr("SD_POW_IFACT_HI", [v >> 64 for v in ifact]))
out.append(arr("SD_POW_IFACT_LO", [v & M64 for v in ifact]))
out.append(arr("SD_POW_EXP2T_HI", [v >> 64 for v in exp2t]))
out.append(arr("SD_POW_EXP2T_LO", [v & M64 for v in exp2t]))
out.append(f"#define SD_POW_INV_LN2_HI (0x{inv_ln2 >> 64:016x}ULL)")
out.append(f"#define SD_POW_INV_LN2_LO (0x{inv_ln2 & M64:016x}ULL)")
out.append(f"#define SD_EXP_LOG2E_HI (0x{log2e_q96 >> 64:016x}ULL)")
out.append(f"#define SD_EXP_LOG2E_LO (0x{log2e_q96 & M64:016x}ULL)")
out.append(f"#define SD_POW_LN2_HI (0x{ln2 >> 64:016x}ULL)")
out.append(f"#define SD_POW_LN2_LO (0x{ln2 & M64:016x}ULL)")
print("\n".join(out))
