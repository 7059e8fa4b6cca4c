"""Generate field_ptx.cuh: Montgomery multiplication and modular add/sub for
the BLS12-381 base field (12 x 32-bit limbs) and scalar field (8 x 32-bit
limbs) as inline-PTX carry chains (mad.lo.cc / madc.hi.cc / addc / subc).

Run:  python gen_field_ptx.py   (rewrites field_ptx.cuh beside this file)

The multiplication is operand-scanning CIOS: for each limb b_i of the second
operand, one asm block adds lo(a*b_i) and hi(a*b_i), computes the Montgomery
quotient m = t0 * (-p^-1 mod 2^32), and adds lo(m*p) and hi(m*p).  Each block
keeps its carry flag local, so no condition code crosses asm statements.  The
modulus words are embedded as immediates.  Intermediate values stay below
2^(32n+32), which the bounds in the comments of field_ptx.cuh document.
"""
import pathlib

P = int("1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab", 16)
R = int("73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001", 16)


def limbs(x, n):
    return [(x >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def gen_field(name, mod, n):
    ml = limbs(mod, n)
    pinv = (-pow(mod, -1, 1 << 32)) % (1 << 32)
    Rm = (1 << (32 * n)) % mod
    R2 = (Rm * Rm) % mod
    out = []
    w = out.append
    w(f"// ---- {name}: {n} x 32-bit limbs, modulus 0x{mod:x}")
    w(f"#define {name.upper()}_NLIMBS {n}")
    w(f"__device__ __constant__ static const uint32_t {name.upper()}_MOD[{n}] = {{{', '.join(f'0x{x:08x}u' for x in ml)}}};")
    w(f"static const uint32_t {name.upper()}_MOD_H[{n}] = {{{', '.join(f'0x{x:08x}u' for x in ml)}}};")
    w(f"static const uint32_t {name.upper()}_ONE_H[{n}] = {{{', '.join(f'0x{x:08x}u' for x in limbs(Rm, n))}}};")
    w(f"static const uint32_t {name.upper()}_R2_H[{n}] = {{{', '.join(f'0x{x:08x}u' for x in limbs(R2, n))}}};")
    w(f"#define {name.upper()}_PINV 0x{pinv:08x}u")
    w(f"#define {name.upper()}_MOD_INIT {{{{{', '.join(f'0x{x:08x}u' for x in ml)}}}}}")
    w(f"#define {name.upper()}_ONE_INIT {{{{{', '.join(f'0x{x:08x}u' for x in limbs(Rm, n))}}}}}")
    w(f"#define {name.upper()}_R2_INIT {{{{{', '.join(f'0x{x:08x}u' for x in limbs(R2, n))}}}}}")
    w("")
    # ---- one CIOS row: t[0..n] (n+1 words, t[n] == 0 on entry) += a*b ; += m*mod ; t[0] becomes 0.
    regs_t = [f"%{i}" for i in range(n + 1)]
    regs_a = [f"%{n + 1 + i}" for i in range(n)]
    reg_b = f"%{2 * n + 1}"
    body = []
    body.append("{ .reg .u32 m;")
    # pass A: lo(a*b)
    body.append(f"mad.lo.cc.u32 {regs_t[0]}, {regs_a[0]}, {reg_b}, {regs_t[0]};")
    for j in range(1, n):
        body.append(f"madc.lo.cc.u32 {regs_t[j]}, {regs_a[j]}, {reg_b}, {regs_t[j]};")
    body.append(f"addc.u32 {regs_t[n]}, 0, 0;")
    # pass B: hi(a*b) into t[1..n]
    body.append(f"mad.hi.cc.u32 {regs_t[1]}, {regs_a[0]}, {reg_b}, {regs_t[1]};")
    for j in range(1, n - 1):
        body.append(f"madc.hi.cc.u32 {regs_t[j + 1]}, {regs_a[j]}, {reg_b}, {regs_t[j + 1]};")
    body.append(f"madc.hi.u32 {regs_t[n]}, {regs_a[n - 1]}, {reg_b}, {regs_t[n]};")
    # quotient
    body.append(f"mul.lo.u32 m, {regs_t[0]}, 0x{pinv:08x};")
    # pass C: lo(m*mod)
    body.append(f"mad.lo.cc.u32 {regs_t[0]}, m, 0x{ml[0]:08x}, {regs_t[0]};")
    for j in range(1, n):
        body.append(f"madc.lo.cc.u32 {regs_t[j]}, m, 0x{ml[j]:08x}, {regs_t[j]};")
    body.append(f"addc.u32 {regs_t[n]}, {regs_t[n]}, 0;")
    # pass D: hi(m*mod) into t[1..n]
    body.append(f"mad.hi.cc.u32 {regs_t[1]}, m, 0x{ml[0]:08x}, {regs_t[1]};")
    for j in range(1, n - 1):
        body.append(f"madc.hi.cc.u32 {regs_t[j + 1]}, m, 0x{ml[j]:08x}, {regs_t[j + 1]};")
    body.append(f"madc.hi.u32 {regs_t[n]}, m, 0x{ml[n - 1]:08x}, {regs_t[n]};")
    body.append("}")
    asm_text = "\\n\\t".join(body)
    w(f"// t[0..{n}] += a*b + m*mod with m = t0*pinv; afterwards t0 == 0 and the value is t[1..{n}].")
    w(f"__device__ __forceinline__ void {name}_cios_row(uint32_t *t, const uint32_t *a, uint32_t b) {{")
    outs = ", ".join(f'"+&r"(t[{i}])' for i in range(n + 1))
    ins = ", ".join(f'"r"(a[{i}])' for i in range(n)) + ', "r"(b)'
    w(f'  asm volatile("{asm_text}" : {outs} : {ins});')
    w("}")
    w("")
    # ---- conditional subtract: r = t >= mod ? t - mod : t  (t < 2*mod)
    body = []
    body.append("{ .reg .u32 d<%d>; .reg .u32 bw; .reg .pred ge;" % n)
    body.append(f"sub.cc.u32 d0, %{n}, 0x{ml[0]:08x};")
    for j in range(1, n):
        body.append(f"subc.cc.u32 d{j}, %{n + j}, 0x{ml[j]:08x};")
    body.append("subc.u32 bw, 0, 0;")
    body.append("setp.eq.u32 ge, bw, 0;")
    for j in range(n):
        body.append(f"selp.u32 %{j}, d{j}, %{n + j}, ge;")
    body.append("}")
    asm_text = "\\n\\t".join(body)
    w(f"__device__ __forceinline__ void {name}_reduce_once(uint32_t *r, const uint32_t *t) {{")
    outs = ", ".join(f'"=&r"(r[{i}])' for i in range(n))
    ins = ", ".join(f'"r"(t[{i}])' for i in range(n))
    w(f'  asm("{asm_text}" : {outs} : {ins});')
    w("}")
    w("")
    # ---- add: r = a + b mod (a,b < mod; sum < 2^(32n) as mod < 2^(32n-1))
    body = []
    body.append("{ .reg .u32 s<%d>; .reg .u32 d<%d>; .reg .u32 bw; .reg .pred ge;" % (n, n))
    body.append(f"add.cc.u32 s0, %{n}, %{2 * n};")
    for j in range(1, n):
        body.append(f"addc.cc.u32 s{j}, %{n + j}, %{2 * n + j};")
    body.append(f"sub.cc.u32 d0, s0, 0x{ml[0]:08x};")
    for j in range(1, n):
        body.append(f"subc.cc.u32 d{j}, s{j}, 0x{ml[j]:08x};")
    body.append("subc.u32 bw, 0, 0;")
    body.append("setp.eq.u32 ge, bw, 0;")
    for j in range(n):
        body.append(f"selp.u32 %{j}, d{j}, s{j}, ge;")
    body.append("}")
    asm_text = "\\n\\t".join(body)
    w(f"__device__ __forceinline__ void {name}_add_raw(uint32_t *r, const uint32_t *a, const uint32_t *b) {{")
    outs = ", ".join(f'"=&r"(r[{i}])' for i in range(n))
    ins = ", ".join(f'"r"(a[{i}])' for i in range(n)) + ", " + ", ".join(f'"r"(b[{i}])' for i in range(n))
    w(f'  asm("{asm_text}" : {outs} : {ins});')
    w("}")
    w("")
    # ---- sub: r = a - b mod
    body = []
    body.append("{ .reg .u32 s<%d>; .reg .u32 bw;" % n)
    body.append(f"sub.cc.u32 s0, %{n}, %{2 * n};")
    for j in range(1, n):
        body.append(f"subc.cc.u32 s{j}, %{n + j}, %{2 * n + j};")
    body.append("subc.u32 bw, 0, 0;")
    # add (mod & bw)
    body.append("{ .reg .u32 k;")
    body.append(f"and.b32 k, bw, 0x{ml[0]:08x};")
    body.append("add.cc.u32 %0, s0, k;")
    for j in range(1, n):
        body.append(f"and.b32 k, bw, 0x{ml[j]:08x};")
        cc = ".cc" if j < n - 1 else ""
        body.append(f"addc{cc}.u32 %{j}, s{j}, k;")
    body.append("}}")
    asm_text = "\\n\\t".join(body)
    w(f"__device__ __forceinline__ void {name}_sub_raw(uint32_t *r, const uint32_t *a, const uint32_t *b) {{")
    w(f'  asm("{asm_text}" : {outs} : {ins});')
    w("}")
    w("")
    return "\n".join(out)


def gen_lazy(name, mod, n):
    """Unreduced sums for short signed sums of reduced values (at most 6 terms
    of [0, mod], so every partial sum stays below 6 mod < 2^(32n)):
    {name}_acc_add (plain add), {name}_from_mod (mod - a) and {name}_csub{k}
    (subtract k*mod when the value is at least k*mod, k = 4, 2, 1), which bring
    a value below 8 mod back to [0, mod)."""
    assert 6 * mod < 1 << (32 * n)
    out = []
    w = out.append
    outs = ", ".join(f'"=&r"(r[{i}])' for i in range(n))
    ins2 = ", ".join(f'"r"(a[{i}])' for i in range(n)) + ", " + ", ".join(f'"r"(b[{i}])' for i in range(n))
    ins1 = ", ".join(f'"r"(a[{i}])' for i in range(n))
    body = [f"add.cc.u32 %0, %{n}, %{2 * n};"]
    for j in range(1, n):
        body.append(f"add{'c.cc' if j < n - 1 else 'c'}.u32 %{j}, %{n + j}, %{2 * n + j};")
    w(f"__device__ __forceinline__ void {name}_acc_add(uint32_t *r, const uint32_t *a, const uint32_t *b) {{")
    w(f'  asm("' + "\\n\\t".join(body) + f'" : {outs} : {ins2});')
    w("}")
    ml = limbs(mod, n)
    body = [f"sub.cc.u32 %0, 0x{ml[0]:08x}, %{n};"]
    for j in range(1, n):
        body.append(f"sub{'c.cc' if j < n - 1 else 'c'}.u32 %{j}, 0x{ml[j]:08x}, %{n + j};")
    w(f"__device__ __forceinline__ void {name}_from_mod(uint32_t *r, const uint32_t *a) {{")
    w(f'  asm("' + "\\n\\t".join(body) + f'" : {outs} : {ins1});')
    w("}")
    for k in (4, 2, 1):
        kl = limbs(k * mod, n)
        body = ["{ .reg .u32 d<%d>; .reg .u32 bw; .reg .pred ge;" % n, f"sub.cc.u32 d0, %{n}, 0x{kl[0]:08x};"]
        for j in range(1, n):
            body.append(f"subc.cc.u32 d{j}, %{n + j}, 0x{kl[j]:08x};")
        body.append("subc.u32 bw, 0, 0;")
        body.append("setp.eq.u32 ge, bw, 0;")
        for j in range(n):
            body.append(f"selp.u32 %{j}, d{j}, %{n + j}, ge;")
        body.append("}")
        w(f"__device__ __forceinline__ void {name}_csub{k}(uint32_t *r, const uint32_t *a) {{")
        w(f'  asm("' + "\\n\\t".join(body) + f'" : {outs} : {ins1});')
        w("}")
    w("")
    return "\n".join(out)


def main():
    text = [
        "// GENERATED by gen_field_ptx.py -- do not edit by hand.",
        "// Inline-PTX carry chains for BLS12-381 Fp (12 limbs) and Fr (8 limbs).",
        "#pragma once",
        "#include <stdint.h>",
        "",
        gen_field("fp", P, 12),
        gen_lazy("fp", P, 12),
        gen_field("fr", R, 8),
    ]
    dst = pathlib.Path(__file__).with_name("field_ptx.cuh")
    dst.write_text("\n".join(text) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    main()
