&HEADING
  modelFile = 'cantilever with prescribed tip deflection'
/
&MECHANISM
  id = 1
  weightTranslation = 0.1
  weightRotation = 1.0
  weightGeneralized = 1.0
/
&TRIAD
  id = 1
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 0.0
  BC = 0 0 0 0 0 0
/
&TRIAD
  id = 2
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 2.0
/
&TRIAD
  id = 3
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 4.0
/
&TRIAD
  id = 4
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 6.0
/
&TRIAD
  id = 5
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 8.0
/
&TRIAD
  id = 6
  nDOFs = 6
  ur = 1.0 0.0 0.0 0.0 0.0 1.0 0.0 0.0 0.0 0.0 1.0 10.0
  BC = 2 1 1 1 1 1
/
&SUP_EL
  id = 7
  numTriads = 2
  triadIds = 1 2
  elPropId = 1
  shadowPosAlg = 1
  refTriad1Id = 1, offset1 = 0.0 0.0 0.0
  refTriad2Id = 2, offset2 = 0.0 0.0 0.0
  refTriad3Id = 1, offset3 = 0.0 2.0 0.0
  supPos = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 7
  triadId = 1
  undPosInSupElSystem = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 7
  triadId = 2
  undPosInSupElSystem = 0.0 0.0 -1.0 2.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&SUP_EL
  id = 8
  numTriads = 2
  triadIds = 2 3
  elPropId = 1
  shadowPosAlg = 1
  refTriad1Id = 2, offset1 = 0.0 0.0 0.0
  refTriad2Id = 3, offset2 = 0.0 0.0 0.0
  refTriad3Id = 2, offset3 = 0.0 2.0 0.0
  supPos = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 2.0
/
&TRIAD_UNDPOS
  supElId = 8
  triadId = 2
  undPosInSupElSystem = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 8
  triadId = 3
  undPosInSupElSystem = 0.0 0.0 -1.0 2.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&SUP_EL
  id = 9
  numTriads = 2
  triadIds = 3 4
  elPropId = 1
  shadowPosAlg = 1
  refTriad1Id = 3, offset1 = 0.0 0.0 0.0
  refTriad2Id = 4, offset2 = 0.0 0.0 0.0
  refTriad3Id = 3, offset3 = 0.0 2.0 0.0
  supPos = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 4.0
/
&TRIAD_UNDPOS
  supElId = 9
  triadId = 3
  undPosInSupElSystem = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 9
  triadId = 4
  undPosInSupElSystem = 0.0 0.0 -1.0 2.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&SUP_EL
  id = 10
  numTriads = 2
  triadIds = 4 5
  elPropId = 1
  shadowPosAlg = 1
  refTriad1Id = 4, offset1 = 0.0 0.0 0.0
  refTriad2Id = 5, offset2 = 0.0 0.0 0.0
  refTriad3Id = 4, offset3 = 0.0 2.0 0.0
  supPos = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 6.0
/
&TRIAD_UNDPOS
  supElId = 10
  triadId = 4
  undPosInSupElSystem = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 10
  triadId = 5
  undPosInSupElSystem = 0.0 0.0 -1.0 2.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&SUP_EL
  id = 11
  numTriads = 2
  triadIds = 5 6
  elPropId = 1
  shadowPosAlg = 1
  refTriad1Id = 5, offset1 = 0.0 0.0 0.0
  refTriad2Id = 6, offset2 = 0.0 0.0 0.0
  refTriad3Id = 5, offset3 = 0.0 2.0 0.0
  supPos = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 8.0
/
&TRIAD_UNDPOS
  supElId = 11
  triadId = 5
  undPosInSupElSystem = 0.0 0.0 -1.0 0.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&TRIAD_UNDPOS
  supElId = 11
  triadId = 6
  undPosInSupElSystem = 0.0 0.0 -1.0 2.0 0.0 1.0 0.0 0.0 1.0 0.0 0.0 0.0
/
&ELEMENT_PROPERTY
  id = 1
  geometry = 0.015393804 0.0004621989652 0.0004621989652 0.0009243979304 2.0 2.0 0.0 0.0
  material = 7850.0 210000000000.0 81395348840.0
/
&MOTION
  id = 30
  triadId = 6
  lDof = 1
  type = 'deflection'
  motionEngineId = 31
  d0 = 0.0
  d1 = 1.0
/
&ENGINE
  id = 31
  functionId = 32
  nArg = 1
  argSensorId = 33
/
&FUNCTION
  id = 32
  type = 'SCALE'
  realDataSize = 1
  realData = 1.0
/
&SENSOR
  id = 33
  type = 'TIME'
/
