"""The Fortran 77 translator that runs the reference on the CPU
(tests/golden/f77.py), checked on small programs of its own: the
arithmetic and control-flow rules the reference runs depend on."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import f77  # noqa: E402


def prog(tmp_path, src, **kw):
    p = tmp_path / "t.f"
    p.write_text(src)
    return f77.Program(str(p), **kw)


def col6(*lines):
    """Fixed-form source: statements start in column 7, labels in 1-5."""
    out = []
    for ln in lines:
        if isinstance(ln, tuple):
            out.append("%-5s %s" % ln)
        elif ln.startswith("&"):
            out.append("     " + ln)
        else:
            out.append("      " + ln)
    return "\n".join(out) + "\n"


def test_real4_literals_and_mixed_precision(tmp_path):
    src = col6("subroutine s(d1, d2, d3, r)",
               "implicit real*8(a-h,o-z)",
               "real*4 r",
               "d1=0.1",
               "d2=0.1d0",
               "d3=2./3.*d2",
               "r=1./3.",
               "return",
               "end")
    P = prog(tmp_path, src)
    c = [f77.cell(0.0) for _ in range(4)]
    P.sub("s")(*c)
    d1, d2, d3, r = (x[0][0] for x in c)
    assert d1 == float(np.float32(0.1)) and d1 != 0.1       # a REAL*4 literal, widened
    assert d2 == 0.1
    assert d3 == float(np.float32(2.0) / np.float32(3.0)) * 0.1
    assert r == float(np.float32(1.0) / np.float32(3.0))


def test_integer_division_powers_and_intrinsics(tmp_path):
    src = col6("subroutine s(i1, i2, i3, x, y)",
               "implicit real*8(a-h,o-z)",
               "i1=-7/2",
               "i2=2**10",
               "i3=mod(-7,3)",
               "x=dble(i1)**2",
               "y=dsqrt(2.d0)*sign(1.d0,-0.d0)",
               "return",
               "end")
    P = prog(tmp_path, src)
    c = [f77.cell(0), f77.cell(0), f77.cell(0), f77.cell(0.0), f77.cell(0.0)]
    P.sub("s")(*c)
    assert [x[0][0] for x in c[:3]] == [-3, 1024, -1]
    assert c[3][0][0] == 9.0
    assert c[4][0][0] == -np.sqrt(2.0)


def test_do_loops_trip_counts_shared_labels_and_exits(tmp_path):
    src = col6("subroutine s(n, i1, i2, i3)",
               "n=0",
               "do 10 i=1,2",
               "do 10 j=1,3",
               "n=n+1",
               ("10", "continue"),
               "do 20 k=1,0",
               "n=n+100",
               ("20", "continue"),
               "i1=k",
               "do 30 k=10,1,-3",
               ("30", "continue"),
               "i2=k",
               "do 40 k=1,10",
               "if(k.eq.3)goto 50",
               ("40", "continue"),
               "k=99",
               ("50", "continue"),
               "i3=k",
               "return",
               "end")
    P = prog(tmp_path, src)
    c = [f77.cell(0) for _ in range(4)]
    P.sub("s")(*c)
    assert [x[0][0] for x in c] == [6, 1, -2, 3]


def test_common_blocks_and_arguments_by_reference(tmp_path):
    src = col6("subroutine a(x)",
               "real*8 x(5), s",
               "common /blk/ s",
               "s=x(1)+x(2)",
               "call b(x(3))",
               "return",
               "end",
               "subroutine b(y)",
               "real*8 y(2), s",
               "common /blk/ s",
               "y(1)=s",
               "y(2)=-1.d0",
               "return",
               "end")
    P = prog(tmp_path, src)
    x = [1.0, 2.0, 0.0, 0.0, 7.0]
    P.sub("a")(f77.ref(x))
    assert x == [1.0, 2.0, 3.0, -1.0, 7.0]      # b wrote a(3), a(4): sequence association
    assert P.common_member("blk", "s")[0] == 3.0


def test_fixed_form_columns_continuations_and_characters(tmp_path):
    src = col6("subroutine s(x, l)",
               "implicit real*8(a-h,o-z)",
               "character*8 ans",
               "logical l",
               "x=1.d0+",
               "&2.d0" + " " * 62 + "+4.d0",
               "ans='no'",
               "l=ans.eq.'no'",
               "return",
               "end")
    P = prog(tmp_path, src)
    c = [f77.cell(0.0), f77.cell(False)]
    P.sub("s")(*c)
    # columns past 72 are dropped: the continuation ends before '+4.d0'
    assert c[0][0][0] == 3.0
    assert c[1][0][0] is True


def test_list_directed_input_deck(tmp_path):
    src = col6("character*20 fname",
               "read*,fname",
               "read*,dt",
               "read*,n",
               "read*,a,b,c",
               "stop",
               "end")
    src = src.replace("      character*20", "      implicit real*8(a-h,o-z)\n      character*20")
    P = prog(tmp_path, src, with_main=True, stdin=["out.dat", "1.d-7", "96", "0.5d0,1.0d0,0.1d0"])
    with pytest.raises(f77.FortranStop):
        P.sub("_main")()
    assert P.input.pos == 4


def test_real4_decimal_rounding_ties():
    # the nearest binary32 of a decimal, ties to even
    assert f77.dec_to_r4("0.1") == float(np.float32(0.1))
    assert f77.dec_to_r4("16777217") == 16777216.0        # halfway: to the even neighbour
    assert f77.dec_to_r4("16777219") == 16777220.0


def test_functions_nested_loop_exits_and_stubs(tmp_path):
    src = col6("subroutine s(n, x)",
               "implicit real*8(a-h,o-z)",
               "n=0",
               "do 10 i=1,5",
               "do 10 j=1,5",
               "n=n+1",
               "if(i*j.eq.6)goto 20",
               ("10", "continue"),
               "n=-1",
               ("20", "continue"),
               "call plot(n)",
               "x=twice(dble(n))",
               "return",
               "end",
               "double precision function twice(a)",
               "implicit real*8(a-h,o-z)",
               "twice=2.d0*a",
               "return",
               "end",
               "subroutine plot(n)",
               "n=12345",
               "return",
               "end")
    P = prog(tmp_path, src, stubs=("plot",))
    c = [f77.cell(0), f77.cell(0.0)]
    P.sub("s")(*c)
    # (i, j) = (2, 3) is the first product 6 in loop order: 5 + 3 iterations; the
    # GOTO leaves both loops and skips n=-1; the stubbed plot leaves n alone
    assert c[0][0][0] == 8
    assert c[1][0][0] == 16.0


def test_replace_takes_a_routine_from_a_sibling_file(tmp_path):
    a = tmp_path / "a.f"
    b = tmp_path / "b.f"
    a.write_text(col6("subroutine top(x)", "real*8 x", "call leaf(x)", "return", "end",
                      "subroutine leaf(x)", "real*8 x", "x=1.d0", "return", "end"))
    b.write_text(col6("subroutine leaf(x)", "real*8 x", "x=2.d0", "return", "end"))
    P = f77.Program(str(a), replace={"leaf": str(b)})
    c = f77.cell(0.0)
    P.sub("top")(c)
    assert c[0][0] == 2.0
