"""Oracle for the ratpoints_gpu point-search path.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module, and only as the checker.  No product code
path imports it.

It restates the reference's behaviour on the CPU:

* ``ModularSieve`` drives ``oracle.c`` (the reference's sieve plan, mask basis
  and word sieve, restated in C) through ctypes and returns the modular
  survivor set of a box (src/sieve_plan.cpp, src/sieve.cu).
* ``exhaustive_output`` is the reference's own independent Python integer
  oracle (tests/test_multi_gpu.py:17-40) restated: every reduced (a, b) of the
  box, exact integer square root, default output format.
* ``square_root`` / ``is_squarefree`` restate ExactPolynomial
  (src/exact_polynomial.cpp:25-42, 44-71) with Python integers and Fractions.
* ``parse_real``, ``parse_command_line`` restate src/command_line.cpp; the
  ``Formatter`` restates src/output_formatter.cpp; ``search`` restates
  PointSearch::run and its helpers (src/point_search.cpp:28-99, 131-146,
  171-240); ``run`` restates main (src/main.cpp:48-85).
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess
import sys
from dataclasses import dataclass, field
from fractions import Fraction
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIBRARY = BUILD_DIR / "liboracle.so"
INT_MAX = 2**31 - 1
LLONG_MAX = 2**63 - 1
MAXIMUM_HEIGHT = (LLONG_MAX - 32) // 2          # command_line.cpp:16-17
MAXIMUM_DEGREE = 100                            # command_line.cpp:15
SQUARE_DENOMINATOR_LIMIT = 46340                # command_line.cpp:357-359


def build(force: bool = False) -> Path:
    """Compile oracle.c into oracle/_build/liboracle.so (plain gcc, -O2)."""
    source = ORACLE_DIR / "oracle.c"
    if (not force and LIBRARY.exists()
            and LIBRARY.stat().st_mtime >= source.stat().st_mtime):
        return LIBRARY
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread",
                    "-o", str(tmp), str(source)], check=True)
    os.replace(tmp, LIBRARY)
    return LIBRARY


_lib = None


def library():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        c_ll, c_int, c_u64 = ctypes.c_longlong, ctypes.c_int, ctypes.c_uint64
        lib.rpo_create.restype = ctypes.c_void_p
        lib.rpo_create.argtypes = [ctypes.POINTER(ctypes.c_char_p), c_int, c_ll]
        lib.rpo_destroy.argtypes = [ctypes.c_void_p]
        lib.rpo_words.restype = c_ll
        lib.rpo_words.argtypes = [ctypes.c_void_p]
        lib.rpo_mask_word.restype = ctypes.c_uint32
        lib.rpo_mask_word.argtypes = [ctypes.c_void_p, c_int, c_int, c_ll]
        lib.rpo_sieve.restype = c_ll
        lib.rpo_sieve.argtypes = [ctypes.c_void_p, c_ll, c_ll, c_int,
                                  ctypes.POINTER(c_ll), ctypes.POINTER(c_int), c_ll,
                                  ctypes.POINTER(c_u64)]
        lib.rpo_sieve_count_mt.restype = c_ll
        lib.rpo_sieve_count_mt.argtypes = [ctypes.c_void_p, c_ll, c_ll, c_int, c_int,
                                           ctypes.POINTER(c_u64)]
        lib.rpo_candidate_primes.argtypes = [ctypes.POINTER(c_int)]
        lib.rpo_select.argtypes = [c_ll, ctypes.POINTER(c_int)]
        lib.rpo_decimal_mod.argtypes = [ctypes.c_char_p, c_int]
        lib.rpo_mod_inverse.restype = c_ll
        lib.rpo_mod_inverse.argtypes = [c_ll, c_ll]
        lib.rpo_affine_mask.argtypes = [c_int, ctypes.POINTER(ctypes.c_char_p), c_int,
                                        ctypes.POINTER(ctypes.c_ubyte)]
        lib.rpo_mix_pair.restype = c_u64
        lib.rpo_mix_pair.argtypes = [c_ll, c_ll]
        _lib = lib
    return _lib


def _c_strings(coefficients):
    array = (ctypes.c_char_p * len(coefficients))()
    for i, text in enumerate(coefficients):
        array[i] = text.encode()
    return array


def candidate_primes():
    out = (ctypes.c_int * 36)()
    library().rpo_candidate_primes(out)
    return list(out)


def selected_primes(denominator):
    """The 32 selected candidate primes for one denominator, largest first."""
    primes = candidate_primes()
    out = (ctypes.c_int * 32)()
    if library().rpo_select(denominator, out) != 0:
        raise ValueError("insufficient denominator sieve primes")
    return [primes[i] for i in out]


MASK64 = (1 << 64) - 1


def mix_pair(a: int, d: int) -> int:
    """Order-independent survivor digest term; same formula as oracle.c."""
    z = ((a & MASK64) * 0x9E3779B97F4A7C15) & MASK64
    z ^= (d << 1) & MASK64
    z ^= 0x632BE59BD9B4E019
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


class ModularSieve:
    """Survivor set of the reference's 32-prime modular sieve for one curve and H."""

    def __init__(self, coefficients, bound):
        self._ctx = None
        self.coefficients = [str(c) for c in coefficients]
        self.bound = int(bound)
        self._strings = _c_strings(self.coefficients)
        self._ctx = library().rpo_create(self._strings, len(self.coefficients), self.bound)
        if not self._ctx:
            raise ValueError("oracle context creation failed")

    def close(self):
        if getattr(self, "_ctx", None):
            library().rpo_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()

    @property
    def words(self):
        return library().rpo_words(self._ctx)

    def mask_word(self, candidate, residue, word):
        return library().rpo_mask_word(self._ctx, candidate, residue, word)

    def count(self, first, last, square=False, threads=1):
        checksum = ctypes.c_uint64(0)
        n = library().rpo_sieve_count_mt(self._ctx, first, last, int(square), threads,
                                         ctypes.byref(checksum))
        if n < 0:
            raise ValueError("oracle sieve failed")
        return n, checksum.value

    def survivors(self, first, last, square=False, cap=1 << 24):
        """Sorted list of (a, d) survivors for parameters first..last."""
        n, _ = self.count(first, last, square)
        if n > cap:
            raise ValueError(f"{n} survivors exceed cap {cap}")
        a = (ctypes.c_longlong * max(n, 1))()
        d = (ctypes.c_int * max(n, 1))()
        checksum = ctypes.c_uint64(0)
        got = library().rpo_sieve(self._ctx, first, last, int(square), a, d, n,
                                  ctypes.byref(checksum))
        if got != n:
            raise ValueError("oracle sieve count changed")
        return [(a[i], d[i]) for i in range(n)]


# ---------------------------------------------------------------------------
# Exact arithmetic (src/exact_polynomial.cpp)


def square_root(coefficients, numerator, denominator):
    """Exact sqrt of F(a, b) = sum c_i a^i b^(n-i) (times b for odd n), or None.

    Restates ExactPolynomial::square_root (exact_polynomial.cpp:25-42): Horner in
    a with an accumulated power of b, one extra factor b when the coefficient
    count is even, and a perfect-square test on the non-negative value.
    """
    coeffs = [int(c) for c in coefficients]
    value = coeffs[-1]
    power = 1
    for i in range(len(coeffs) - 2, -1, -1):
        value *= numerator
        power *= denominator
        value += coeffs[i] * power
    if len(coeffs) % 2 == 0:
        value *= denominator
    if value < 0:
        return None
    root = math.isqrt(value)
    return root if root * root == value else None


def is_squarefree(coefficients):
    """gcd(f, f') over Q is a nonzero constant (exact_polynomial.cpp:44-71)."""
    poly = [Fraction(int(c)) for c in coefficients]
    derivative = [poly[i] * i for i in range(1, len(poly))]

    def trim(p):
        while p and p[-1] == 0:
            p.pop()

    trim(derivative)
    while derivative:
        remainder = list(poly)
        while len(remainder) >= len(derivative):
            shift = len(remainder) - len(derivative)
            factor = remainder[-1] / derivative[-1]
            for i, c in enumerate(derivative):
                remainder[i + shift] -= factor * c
            trim(remainder)
        poly, derivative = derivative, remainder
    return len(poly) == 1


def exhaustive_output(coefficients_text, height, first, last):
    """The reference's independent Python oracle (tests/test_multi_gpu.py:17-40)."""
    coeff = list(map(int, coefficients_text.split()))
    degree = len(coeff) - 1
    output = []

    def append(a, value, b):
        if value < 0:
            return
        root = math.isqrt(value)
        if root * root != value:
            return
        output.append(f"({a} : {root} : {b})\n")
        if root:
            output.append(f"({a} : {-root} : {b})\n")

    append(1, 0 if degree % 2 else coeff[-1], 0)
    for b in range(first, last + 1):
        for a in range(-height, height + 1):
            if math.gcd(a, b) != 1:
                continue
            value = sum(c * a ** i * b ** (degree - i) for i, c in enumerate(coeff))
            append(a, value * (b if degree % 2 else 1), b)
    return "".join(output).encode()


# ---------------------------------------------------------------------------
# Command line (src/command_line.cpp)


class UsageError(Exception):
    pass


def parse_positive(text, name):
    """strtoll semantics: leading blanks, optional sign, digits, nothing after."""
    s = text
    i = 0
    while i < len(s) and s[i] in " \t\n\v\f\r":
        i += 1
    j = i
    if j < len(s) and s[j] in "+-":
        j += 1
    k = j
    while k < len(s) and s[k].isdigit() and s[k] in "0123456789":
        k += 1
    if k == j or k != len(s):
        raise UsageError(f"{name} must be positive")
    value = int(s[i:k])
    if value > LLONG_MAX or value < -LLONG_MAX - 1 or value < 1:
        raise UsageError(f"{name} must be positive")
    return value


def parse_positive_int(text, name):
    value = parse_positive(text, name)
    if value > INT_MAX:
        raise UsageError(f"{name} exceeds GPU limit")
    return value


def parse_real(text, name):
    """Exact decimal with optional fraction and exponent (command_line.cpp:39-108)."""
    i = 0
    negative = False
    if i < len(text) and text[i] in "+-":
        negative = text[i] == "-"
        i += 1
    digits = ""
    fractional = 0
    saw_digit = False
    while i < len(text) and "0" <= text[i] <= "9":
        digits += text[i]
        i += 1
        saw_digit = True
    if i < len(text) and text[i] == ".":
        i += 1
        start = len(digits)
        while i < len(text) and "0" <= text[i] <= "9":
            digits += text[i]
            i += 1
            saw_digit = True
        fractional = len(digits) - start
    exponent = 0
    exponent_negative = False
    if i < len(text) and text[i] in "eE":
        i += 1
        if i < len(text) and text[i] in "+-":
            exponent_negative = text[i] == "-"
            i += 1
        start = i
        while i < len(text) and "0" <= text[i] <= "9":
            digit = ord(text[i]) - 48
            i += 1
            if exponent > (10000 - digit) // 10:
                raise UsageError(f"{name} exponent is too large")
            exponent = exponent * 10 + digit
        if i == start:
            raise UsageError(f"{name} must be real")
    if not saw_digit or i != len(text):
        raise UsageError(f"{name} must be real")
    if exponent_negative:
        exponent = -exponent
    numerator = int(digits) if digits else 0
    if negative:
        numerator = -numerator
    scale = fractional - exponent
    return Fraction(numerator, 10 ** scale) if scale >= 0 else Fraction(numerator * 10 ** -scale)


def _is_integer(text):
    index = 1 if text[:1] in ("-", "+") else 0
    if index == len(text):
        return False
    return all("0" <= c <= "9" for c in text[index:])


def _is_zero(text):
    index = 1 if text[:1] in ("-", "+") else 0
    return all(c == "0" for c in text[index:])


def split_coefficients(text):
    out = []
    for token in text.split():
        if token.startswith("+"):
            token = token[1:]
        out.append(token)
    return out


def parse_device_selection(text):
    """--devices syntax (src/gpu_devices.cpp:21-53); [] means all."""
    if text == "all":
        return []
    ids = []
    start = 0
    while start < len(text):
        end = text.find(",", start)
        if end == -1:
            end = len(text)
        if end == start:
            raise UsageError("empty GPU ID in --devices")
        value = 0
        for c in text[start:end]:
            if not "0" <= c <= "9" or value > (INT_MAX - (ord(c) - 48)) // 10:
                raise UsageError("--devices requires all or comma-separated nonnegative GPU IDs")
            value = value * 10 + ord(c) - 48
        if value in ids:
            raise UsageError("duplicate GPU ID in --devices")
        ids.append(value)
        start = end + 1
    if not ids or text.endswith(","):
        raise UsageError("--devices requires all or a nonempty GPU list")
    return ids


def validate_coefficients(coefficients):
    if len(coefficients) < 2 or len(coefficients) > MAXIMUM_DEGREE + 1:
        raise UsageError("supported polynomial degrees are 1 through 100")
    for c in coefficients:
        if not _is_integer(c):
            raise UsageError("coefficients must be decimal integers")
    if _is_zero(coefficients[-1]):
        raise UsageError("leading coefficient must be nonzero")


@dataclass
class Interval:
    lower: Fraction | None   # None = -infinity
    upper: Fraction | None   # None = +infinity


@dataclass
class Options:
    coefficients: list = field(default_factory=list)
    height: int = 0
    first: int = 1
    last: int = 0
    intervals: list = field(default_factory=list)
    include_infinity: bool = True
    devices: list | None = None
    batch_size: int = 1 << 16
    square: bool = False
    print_points: bool = True
    print_y: bool = True
    format: str = ""
    before: str = ""
    between: str = ""
    after: str = ""
    quiet: bool = False
    verbose: bool = False
    stop_after_first: bool = False


USAGE = "Usage: ratpoints_gpu 'c0 c1 ... cn' HEIGHT [OPTIONS]"


def parse_command_line(argv):
    """argv[0] is the program name (command_line.cpp:336-366, 166-286)."""
    if len(argv) < 3:
        raise UsageError(USAGE)
    o = Options()
    o.coefficients = split_coefficients(argv[1])
    o.height = parse_positive(argv[2], "maximum height")
    if o.height > MAXIMUM_HEIGHT:
        raise UsageError("maximum height exceeds safe GPU limit")
    o.last = min(o.height, INT_MAX)
    index = 3
    pending = None
    has_pending = False

    def argument(option):
        nonlocal index
        if index >= len(argv):
            raise UsageError(f"{option} requires an argument")
        index += 1
        return argv[index - 1]

    while index < len(argv):
        option = argv[index]
        index += 1
        if option == "-dl":
            o.first = parse_positive_int(argument(option), "lower denominator")
        elif option == "-du":
            o.last = parse_positive_int(argument(option), "upper denominator")
        elif option == "-l":
            if has_pending:
                raise UsageError("interval lower bound without upper bound")
            pending = parse_real(argument(option), "interval lower bound")
            has_pending = True
        elif option == "-u":
            upper = parse_real(argument(option), "interval upper bound")
            if has_pending and pending > upper:
                raise UsageError("interval lower bound exceeds upper bound")
            if o.intervals and (not has_pending or o.intervals[-1].upper is None
                                or pending < o.intervals[-1].upper):
                raise UsageError("search intervals must be ordered")
            o.intervals.append(Interval(pending if has_pending else None, upper))
            has_pending = False
        elif option == "-i":
            o.include_infinity = False
        elif option == "-I":
            o.include_infinity = True
        elif option == "-y":
            o.print_y = False
        elif option == "-Y":
            o.print_y = True
        elif option == "-z":
            o.print_points = False
        elif option == "-Z":
            o.print_points = True
        elif option == "-f":
            o.format = argument(option)
        elif option == "-fs":
            o.before = argument(option)
        elif option == "-fm":
            o.between = argument(option)
        elif option == "-fe":
            o.after = argument(option)
        elif option == "--devices":
            o.devices = parse_device_selection(argument(option))
        elif option == "--batch-size":
            o.batch_size = parse_positive_int(argument(option), "denominator batch size")
            if o.batch_size > 1 << 16:
                raise UsageError("--batch-size must not exceed 65536")
        elif option == "--square-denominators":
            o.square = True
        elif option == "-q":
            o.quiet = True
        elif option == "-v":
            o.verbose = True
        elif option == "-1":
            o.stop_after_first = True
        elif option in ("-s", "-k", "-K", "-j", "-J"):
            pass
        else:
            raise UsageError(f"unsupported ratpoints option: {option}")
    if has_pending:
        o.intervals.append(Interval(pending, None))
    if o.last > o.height:
        o.last = o.height
    if o.square and o.last > SQUARE_DENOMINATOR_LIMIT:
        o.last = SQUARE_DENOMINATOR_LIMIT
    if o.first > o.last:
        raise UsageError("empty denominator range")
    validate_coefficients(o.coefficients)
    return o


def accepts(intervals, numerator, denominator):
    """Closed-interval union filter (point_search.cpp:131-146)."""
    if not intervals:
        return True
    x = Fraction(numerator, denominator)
    for iv in intervals:
        if (iv.lower is None or x >= iv.lower) and (iv.upper is None or x <= iv.upper):
            return True
    return False


# ---------------------------------------------------------------------------
# Output (src/output_formatter.cpp)

ESCAPED_PERCENT = "\x01"


def decode(text):
    out = []
    i = 0
    while i < len(text):
        c = text[i]
        if c != "\\" or i + 1 == len(text):
            out.append(c)
            i += 1
            continue
        e = text[i + 1]
        i += 2
        if e == "n":
            out.append("\n")
        elif e == "t":
            out.append("\t")
        elif e == "%":
            out.append(ESCAPED_PERCENT)
        else:
            out.append("\\" + e)
    return "".join(out)


class Formatter:
    def __init__(self, o: Options):
        self.print_points = o.print_points
        self.print_y = o.print_y
        fmt = o.format if o.format else ("(%x : %y : %z)\\n" if o.print_y else "(%x : %z)\\n")
        self.format = decode(fmt)
        self.before = decode(o.before)
        self.between = decode(o.between)
        self.after = decode(o.after)
        self.emitted = False
        self.out = []
        if self.print_points:
            self.out.append(self.before)

    def write_point(self, numerator, ordinate, denominator):
        if not self.print_points:
            return
        if self.emitted:
            self.out.append(self.between)
        f = self.format
        s = []
        i = 0
        while i < len(f):
            if f[i] != "%" or i + 1 == len(f):
                s.append(f[i])
                i += 1
                continue
            m = f[i + 1]
            if m == "x":
                s.append(str(numerator))
            elif m == "y" and self.print_y:
                s.append(ordinate)
            elif m == "z":
                s.append(str(denominator))
            else:
                s.append("%" + m)
            i += 2
        self.out.append("".join(s).replace(ESCAPED_PERCENT, "%"))
        self.emitted = True

    def point_pair(self, numerator, ordinate, denominator, include_conjugate=True):
        self.write_point(numerator, ordinate, denominator)
        if include_conjugate and self.print_y and ordinate != "0":
            self.write_point(numerator, "-" + ordinate, denominator)

    def finish(self):
        self.out.append(self.after)

    def text(self):
        return "".join(self.out)


# ---------------------------------------------------------------------------
# Search (src/point_search.cpp) and main (src/main.cpp)


@dataclass
class Metrics:
    denominators: int = 0
    survivors: int = 0
    exact_survivors: int = 0
    words: int = 0


def verified_points(coefficients, survivors):
    """gcd(a, d) = 1 then exact square root (point_search.cpp:48-60), sorted by (d, a)."""
    points = []
    for a, d in survivors:
        if math.gcd(a, d) != 1:
            continue
        root = square_root(coefficients, a, d)
        if root is not None:
            points.append((a, root, d))
    points.sort(key=lambda p: (p[2], p[0]))
    return points


def search(o: Options, callback):
    """PointSearch::run for one device (point_search.cpp:171-240).

    Infinity first, then batches of ``batch_size`` parameters in order; each
    batch's verified points in (d, a) order go through the interval filter and
    the callback, which returns False to stop.
    """
    m = Metrics()
    if o.include_infinity:
        root = square_root(o.coefficients, 1, 0)
        if root is not None and not callback(1, str(root), 0):
            return m
    sieve = ModularSieve(o.coefficients, o.height)
    try:
        m.words = sieve.words
        first = o.first
        while first <= o.last:
            last = min(o.last, first + o.batch_size - 1)
            survivors = sieve.survivors(first, last, o.square)
            points = verified_points(o.coefficients, survivors)
            m.denominators += last - first + 1
            m.survivors += len(survivors)
            m.exact_survivors += len(points)
            first = last + 1
            for a, y, d in points:
                if accepts(o.intervals, a, d) and not callback(a, str(y), d):
                    return m
    finally:
        sieve.close()
    return m


def run(argv, env=None):
    """Restated main(): returns (exit_code, stdout_bytes, stderr_text, metrics).

    ``--devices`` lists naming a GPU other than 0 are rejected as on a host
    with one visible GPU.  The metrics dict holds the integer fields of
    the ``-v`` line that do not depend on timing.
    """
    env = os.environ if env is None else env
    if len(argv) == 1:
        return 1, b"", "help", None
    if len(argv) == 2 and argv[1] in ("--help", "--list-devices"):
        return 0, b"", "", None
    try:
        o = parse_command_line(argv)
        if not is_squarefree(o.coefficients):
            raise UsageError("polynomial is not squarefree")
        if o.devices and any(i != 0 for i in o.devices):
            raise UsageError(f"GPU ID {max(o.devices)} is not visible; run --list-devices "
                             "(IDs are CUDA-visible ordinals)")
        fmt = Formatter(o)

        def callback(a, y, d):
            fmt.point_pair(a, y, d, not o.stop_after_first)
            return not o.stop_after_first

        m = search(o, callback)
        fmt.finish()
        metrics = None
        if env.get("RATPOINTS_GPU_BENCHMARK") is not None or (o.verbose and not o.quiet):
            metrics = {"denominators": m.denominators, "words": m.words,
                       "survivors": m.survivors, "exact_survivors": m.exact_survivors}
        return 0, fmt.text().encode(), "", metrics
    except UsageError as error:
        return 1, b"", str(error), None


if __name__ == "__main__":  # pragma: no cover - manual use
    code, out, err, metrics = run(sys.argv)
    sys.stdout.buffer.write(out)
    if err:
        print(err, file=sys.stderr)
    if metrics:
        print(" ".join(f"{k}={v}" for k, v in metrics.items()), file=sys.stderr)
    sys.exit(code)
