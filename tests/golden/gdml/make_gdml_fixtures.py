"""Write the GDML test geometry tests/golden/gdml/detector.gdml (deterministic; run from the
repository root: python tests/golden/gdml/make_gdml_fixtures.py).

A small detector exercising every solid the reader supports and the GDML conventions it
must follow: mm, cm and m lengths, deg and rad angles, named constants, <define>d positions
and rotations used by reference (positionref/rotationref) and inline ones, a boolean
subtraction whose second solid is placed with a rotation, and nested placements:

  world box (m)
    barrel tube with 6 rings x 24 box modules, each rotated about z
    two endcap polycones (cm z planes) with 8 Trd wedges each; one endcap flipped about x
    a polyhedra holder with two tilted, sheared trapezoids
    a torus ring, a phi-cut cone, and box-minus-rotated-tube
"""
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def detector():
    L = []
    a = L.append
    a('<?xml version="1.0"?>')
    a('<!-- generated by make_gdml_fixtures.py -->')
    a('<gdml xmlns:xsi="http://www.w3.org/2001/XMLSchema-instance">')
    a('  <define>')
    a('    <constant name="RING_R" value="400"/>')
    a('    <constant name="NMOD" value="24"/>')
    a('    <position name="endcap_pos" z="100" unit="cm"/>')
    a('    <position name="endcap_neg" z="-1" unit="m"/>')
    a('    <rotation name="flip" x="180" unit="deg"/>')
    a('    <rotation name="tilt" z="0.5235987755982988"/>')
    a('  </define>')
    a('  <materials/>')
    a('  <solids>')
    a('    <box name="world_s" x="3" y="3" z="4" lunit="m"/>')
    a('    <tube name="barrel_s" rmin="300" rmax="500" z="1500" startphi="0" deltaphi="360" aunit="deg" lunit="mm"/>')
    a('    <box name="module_s" x="20" y="60" z="200"/>')
    a('    <polycone name="endcap_s" startphi="0" deltaphi="360" aunit="deg" lunit="cm">')
    a('      <zplane z="-10" rmin="10" rmax="55"/>')
    a('      <zplane z="0" rmin="10" rmax="60"/>')
    a('      <zplane z="10" rmin="12" rmax="60"/>')
    a('    </polycone>')
    a('    <trd name="wedge_s" x1="80" x2="40" y1="60" y2="30" z="150" lunit="mm"/>')
    a('    <polyhedra name="holder_s" startphi="0" deltaphi="360" numsides="6" aunit="deg" lunit="mm">')
    a('      <zplane z="-150" rmin="0" rmax="200"/>')
    a('      <zplane z="150" rmin="0" rmax="200"/>')
    a('    </polyhedra>')
    a('    <trap name="trap_s" z="100" theta="5" phi="10" y1="80" x1="60" x2="70" alpha1="5" y2="80" x3="60" '
      'x4="70" alpha2="5" aunit="deg" lunit="mm"/>')
    a('    <torus name="ring_s" rmin="0" rmax="30" rtor="1000" startphi="0" deltaphi="6.283185307179586" '
      'aunit="rad" lunit="mm"/>')
    a('    <cone name="cone_s" rmin1="0" rmax1="100" rmin2="0" rmax2="200" z="300" startphi="0" deltaphi="270" '
      'aunit="deg"/>')
    a('    <box name="block_s" x="200" y="200" z="200"/>')
    a('    <tube name="hole_s" rmin="0" rmax="50" z="300" deltaphi="360" aunit="deg"/>')
    a('    <subtraction name="drilled_s">')
    a('      <first ref="block_s"/>')
    a('      <second ref="hole_s"/>')
    a('      <position name="hole_pos" x="3" unit="cm"/>')
    a('      <rotation name="hole_rot" x="90" unit="deg"/>')
    a('    </subtraction>')
    a('  </solids>')
    a('  <structure>')
    a('    <volume name="module"><materialref ref="Si"/><solidref ref="module_s"/></volume>')
    a('    <volume name="barrel">')
    a('      <solidref ref="barrel_s"/>')
    k = 0
    for ring in range(6):
        z = -625.0 + 250.0 * ring
        for j in range(24):
            ph = 2.0 * math.pi * j / 24
            a('      <physvol name="mod%d" copynumber="%d"><volumeref ref="module"/>' % (k, k))
            a('        <position name="mod%d_p" x="%.17g" y="%.17g" z="%.17g"/>'
              % (k, 400.0 * math.cos(ph), 400.0 * math.sin(ph), z))
            a('        <rotation name="mod%d_r" z="%.17g" unit="deg"/>' % (k, -360.0 * j / 24))
            a('      </physvol>')
            k += 1
    a('    </volume>')
    a('    <volume name="wedge"><solidref ref="wedge_s"/></volume>')
    a('    <volume name="endcap">')
    a('      <solidref ref="endcap_s"/>')
    for j in range(8):
        ph = 2.0 * math.pi * (j + 0.5) / 8
        a('      <physvol><volumeref ref="wedge"/>')
        a('        <position name="w%d_p" x="%.17g" y="%.17g" unit="cm"/>' % (j, 35.0 * math.cos(ph), 35.0 * math.sin(ph)))
        a('        <rotation name="w%d_r" z="%.17g"/>' % (j, -ph))
        a('      </physvol>')
    a('    </volume>')
    a('    <volume name="trap"><solidref ref="trap_s"/></volume>')
    a('    <volume name="holder">')
    a('      <solidref ref="holder_s"/>')
    a('      <physvol><volumeref ref="trap"/><position name="t0" x="-90" z="-60"/><rotationref ref="tilt"/></physvol>')
    a('      <physvol><volumeref ref="trap"/><position name="t1" x="90" z="60"/><rotationref ref="tilt"/></physvol>')
    a('    </volume>')
    a('    <volume name="ring"><solidref ref="ring_s"/></volume>')
    a('    <volume name="cone"><solidref ref="cone_s"/></volume>')
    a('    <volume name="drilled"><solidref ref="drilled_s"/></volume>')
    a('    <volume name="World">')
    a('      <solidref ref="world_s"/>')
    a('      <physvol name="barrel_pv"><volumeref ref="barrel"/></physvol>')
    a('      <physvol><volumeref ref="endcap"/><positionref ref="endcap_pos"/></physvol>')
    a('      <physvol><volumeref ref="endcap"/><positionref ref="endcap_neg"/><rotationref ref="flip"/></physvol>')
    a('      <physvol><volumeref ref="holder"/><position name="h_p" x="1.1" y="1.1" z="1.4" unit="m"/></physvol>')
    a('      <physvol><volumeref ref="ring"/><position name="r_p" z="1500"/></physvol>')
    a('      <physvol><volumeref ref="cone"/><position name="c_p" x="-1000" y="-1000" z="-1400"/>'
      '<rotation name="c_r" y="0.3"/></physvol>')
    a('      <physvol><volumeref ref="drilled"/><position name="d_p" x="1000" y="-1000"/></physvol>')
    a('    </volume>')
    a('  </structure>')
    a('  <setup name="Default" version="1.0"><world ref="World"/></setup>')
    a('</gdml>')
    return "\n".join(L) + "\n"


if __name__ == "__main__":
    with open(os.path.join(HERE, "detector.gdml"), "w") as f:
        f.write(detector())
