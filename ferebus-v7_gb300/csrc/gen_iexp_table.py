"""Generate iexp_table.h: constants of the engine's fixed-point exponential.

exp(x), x <= 0, is evaluated on the integer pipes as 2^-|y| with
|y| = |x| log2(e) held with 64 fractional bits, m = ceil(|y|),
g = m - |y| = j/256 + s:  2^-|y| = 2^-m 2^(j/256) exp(s ln2).
Constants (computed here with mpmath at 80 digits, each rounded once):

  L2E_HI, L2E_LO  floor(log2(e) 2^127) as two 64-bit words
  L2E64           nearest integer to log2(e) 2^63
  LN2             nearest integer to ln2 2^64
  C2 .. C5        nearest integers to 2^63 / k!  (Taylor coefficients of exp)
  table[j]        nearest integer to 2^(j/256) 2^63, j = 0..255
  table1024[j]    nearest integer to 2^(j/1024) 2^63, j = 0..1023 (the
                  kernel-matrix build's variant)
  fine1024[k]     nearest integer to (2^(k/2^20) - 1) 2^64, k = 0..1023 (its
                  second table: the rest below 2^-20 needs a degree-2
                  polynomial only)

Run: python gen_iexp_table.py > iexp_table.h
"""
import mpmath as mp

mp.mp.dps = 80
L = int(mp.floor(mp.mpf(2) ** 127 / mp.log(2)))
LN2 = int(mp.nint(mp.log(2) * mp.mpf(2) ** 64))
C = {k: int(mp.nint(mp.mpf(2) ** 63 / mp.factorial(k))) for k in range(2, 6)}
tab = [int(mp.nint(mp.mpf(2) ** (mp.mpf(j) / 256 + 63))) for j in range(256)]
tab1024 = [int(mp.nint(mp.mpf(2) ** (mp.mpf(j) / 1024 + 63))) for j in range(1024)]
fine1024 = [int(mp.nint((mp.mpf(2) ** (mp.mpf(k) / 2 ** 20) - 1) * mp.mpf(2) ** 64)) for k in range(1024)]
L2E64 = int(mp.nint(mp.mpf(2) ** 63 / mp.log(2)))
print("// Generated by gen_iexp_table.py (constants of the fixed-point exponential).")
print("#pragma once")
print(f"#define IEXP_L2E_HI 0x{L >> 64:016x}ULL  // floor(log2(e) 2^127), high word")
print(f"#define IEXP_L2E_LO 0x{L & ((1 << 64) - 1):016x}ULL  // low word")
print(f"#define IEXP_L2E64 0x{L2E64:016x}ULL  // log2(e) 2^63, nearest")
print(f"#define IEXP_LN2 0x{LN2:016x}ULL     // ln2 2^64")
for k in range(2, 6):
    print(f"#define IEXP_C{k} 0x{C[k]:016x}ULL      // 2^63 / {k}!")
print("// 2^(j/256) 2^63")
print("static __device__ const unsigned long long g_iexp_tab[256] = {")
for j in range(0, 256, 4):
    print("    " + ", ".join(f"0x{t:016x}ULL" for t in tab[j:j + 4]) + ",")
print("};")
print("// 2^(j/1024) 2^63")
print("static __device__ const unsigned long long g_iexp_tab1024[1024] = {")
for j in range(0, 1024, 4):
    print("    " + ", ".join(f"0x{t:016x}ULL" for t in tab1024[j:j + 4]) + ",")
print("};")
print("// (2^(k/2^20) - 1) 2^64")
print("static __device__ const unsigned long long g_iexp_fine1024[1024] = {")
for k in range(0, 1024, 4):
    print("    " + ", ".join(f"0x{t:016x}ULL" for t in fine1024[k:k + 4]) + ",")
print("};")
