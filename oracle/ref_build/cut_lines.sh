#!/bin/sh
# cut_lines.sh FILE FIRST LAST EXPECTED_FIRST_LINE OUT
# Copies lines FIRST..LAST of FILE (a reference source, read in place) to OUT under the
# build directory and checks that the cut starts with EXPECTED_FIRST_LINE and ends with
# a closing brace, so a different reference tree fails loudly instead of compiling
# something else.
set -e
mkdir -p "$(dirname "$5")"
sed -n "$2,$3p" "$1" > "$5"
if ! head -n 1 "$5" | grep -qF -- "$4"; then echo "cut_lines: unexpected first line in $5" >&2; rm -f "$5"; exit 1; fi
if ! tail -n 1 "$5" | grep -qx '}'; then echo "cut_lines: unexpected last line in $5" >&2; rm -f "$5"; exit 1; fi
