"""Derive the constants of the deterministic FP64 sin/cos from first principles.

Each constant is the double nearest to pi/2 (split in three parts), 2/pi or
(+-)1/n!. Run with mpmath available; the output is pasted verbatim into
devmath.cuh (and the oracle's copy of the same method). tanh and expm1 use the
published constants of their method instead (devmath.cuh).
"""
import mpmath as mp

mp.mp.prec = 300


def rn(x):
    return float(x)


def main():
    pio2 = mp.pi / 2
    p1 = rn(pio2)
    p2 = rn(pio2 - p1)
    p3 = rn(pio2 - p1 - p2)
    print(f"PIO2_1 {p1.hex()}\nPIO2_2 {p2.hex()}\nPIO2_3 {p3.hex()}")
    print(f"2_OVER_PI {rn(2 / mp.pi).hex()}")
    for n in range(3, 18, 2):
        print(f"S{n} {rn((-1) ** ((n - 1) // 2) / mp.factorial(n)).hex()}")
    for n in range(4, 19, 2):
        print(f"C{n} {rn((-1) ** (n // 2) / mp.factorial(n)).hex()}")


if __name__ == "__main__":
    main()
