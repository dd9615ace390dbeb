"""Write vesper_twiddles.cuh: exp(-2 pi i j / N) for j < N, float32, for every
composite N <= 32 whose prime factors are 2, 3, 5, 7, 11, 13 (the register
DFT sizes of vesper_regfft.cuh).  Run: python gen_twiddles.py > vesper_twiddles.cuh"""
import math


def sizes():
    out = []
    for n in range(4, 33):
        m = n
        for p in (2, 3, 5, 7, 11, 13):
            while m % p == 0:
                m //= p
        if m == 1 and n not in (5, 7, 11, 13):
            out.append(n)
    return out


def main():
    ns = sizes()
    print("// Generated by gen_twiddles.py: exp(-2 pi i j / N), j < N, float32.")
    print("#pragma once")
    print("namespace vg {")
    off = 0
    offs = {}
    vals = []
    for n in ns:
        offs[n] = off
        for j in range(n):
            a = -2.0 * math.pi * j / n
            vals.append((math.cos(a), math.sin(a)))
        off += n
    print(f"__constant__ float2 c_rtw[{off}] = {{")
    for c, s in vals:
        print(f"    {{{c!r}f, {s!r}f}},")
    print("};")
    print("template <int N> __host__ __device__ constexpr int rtw_off() {")
    print("    return " + " : ".join(f"N == {n} ? {offs[n]}" for n in ns) + " : -1;")
    print("}")
    print("}  // namespace vg")


if __name__ == "__main__":
    main()
