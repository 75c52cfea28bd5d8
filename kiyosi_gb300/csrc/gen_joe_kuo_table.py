"""Regenerates joe_kuo_6_21201.inc, the Sobol primitive-polynomial table.

The table is the published new-joe-kuo-6.21201 data set of Stephen Joe and Frances Kuo
(search criterion 6, https://web.maths.unsw.edu.au/~fkuo/sobol/), BSD-style licence
reproduced in the generated file.  kiyosi bundles the same data set
(crates/kiyosi/src/engines/monte_carlo/sobol_joe_kuo.rs); this script reads the numbers
out of that bundle so that both builds use identical direction numbers, and writes
them in this project's own layout: one record per dimension >= 1, each record
`degree, coefficients, m_1 .. m_degree`, flattened into a uint32 array.

Usage: python gen_joe_kuo_table.py <path to sobol_joe_kuo.rs> [out.inc]
"""
import os
import re
import sys

LICENCE = """\
 * Joe-Kuo Sobol direction numbers, new-joe-kuo-6.21201 (search criterion 6).
 * Source: https://web.maths.unsw.edu.au/~fkuo/sobol/
 *
 * Copyright (c) 2008, Frances Y. Kuo and Stephen Joe
 * All rights reserved.
 *
 * Redistribution and use in source and binary forms, with or without
 * modification, are permitted provided that the following conditions are met:
 *
 *     * Redistributions of source code must retain the above copyright
 *       notice, this list of conditions and the following disclaimer.
 *
 *     * Redistributions in binary form must reproduce the above copyright
 *       notice, this list of conditions and the following disclaimer in the
 *       documentation and/or other materials provided with the distribution.
 *
 *     * Neither the names of the copyright holders nor the names of the
 *       University of New South Wales and the University of Waikato
 *       and its contributors may be used to endorse or promote products derived
 *       from this software without specific prior written permission.
 *
 * THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS ``AS IS'' AND ANY
 * EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO, THE IMPLIED
 * WARRANTIES OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE ARE
 * DISCLAIMED. IN NO EVENT SHALL THE COPYRIGHT HOLDERS BE LIABLE FOR ANY
 * DIRECT, INDIRECT, INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL DAMAGES
 * (INCLUDING, BUT NOT LIMITED TO, PROCUREMENT OF SUBSTITUTE GOODS OR SERVICES;
 * LOSS OF USE, DATA, OR PROFITS; OR BUSINESS INTERRUPTION) HOWEVER CAUSED AND
 * ON ANY THEORY OF LIABILITY, WHETHER IN CONTRACT, STRICT LIABILITY, OR TORT
 * (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN ANY WAY OUT OF THE USE OF THIS
 * SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH DAMAGE.
"""


def main():
    src = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(
        os.path.dirname(os.path.abspath(__file__)), "joe_kuo_6_21201.inc")
    text = open(src).read()
    body = text[text.index("= [") + 3: text.rindex("]")]
    values = [int(v) for v in re.findall(r"\d+", body)]
    # Validate the record structure: degree, coefficients, degree initial numbers.
    i = records = 0
    while i < len(values):
        degree = values[i]
        assert 1 <= degree <= 18, degree
        i += degree + 2
        records += 1
    assert i == len(values) and records == 21200, (i, len(values), records)
    with open(out, "w") as f:
        f.write("/*\n" + LICENCE + " *\n * Generated by gen_joe_kuo_table.py: %d records "
                "(dimensions 2..21201), %d words.\n */\n" % (records, len(values)))
        f.write("#define KGPU_JOE_KUO_RECORDS %d\n#define KGPU_JOE_KUO_WORDS %d\n"
                % (records, len(values)))
        f.write("static const uint32_t kgpu_joe_kuo_table[KGPU_JOE_KUO_WORDS] = {\n")
        for start in range(0, len(values), 24):
            f.write(",".join(str(v) for v in values[start:start + 24]) + ",\n")
        f.write("};\n")


if __name__ == "__main__":
    main()
