{
   /* Emitters of every kind the GPU path takes: a ceiling plane given by vertices (two emitting
    * culled Triangles), a transformed emitting triangle shape with its own uvs, an emitting OBJ
    * mesh (one mesh light over its eight triangles) and a unit-plane light. */
   "scenefile" : {
      "renderer" : { "type" : "pathTracer", "noSuperSamples" : 16, "noDirectSamples" : 4,
                     "maxDepth" : 4, "rrStartDepth" : 2, },
      "camera" : { "type" : "pinhole", "eye" : [ 0, 1, 3.5 ], "look" : [ 0, 0, -1 ], "up" : [ 0, 1, 0 ],
                   "heightAngle" : 45, },
      "output" : { "width" : 40, "height" : 40, },
      "scene" : {
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.7, 0.7, 0.7 ], },
            "plane" : { "vertices" : [ -1, 0, 1,   1, 0, 1,   1, 0, -1,   -1, 0, -1 ], },
            "plane" : { "vertices" : [ -1, 0, -1,   1, 0, -1,   1, 2, -1,   -1, 2, -1 ], },
            "plane" : { "vertices" : [ -1, 0, 1,   -1, 0, -1,   -1, 2, -1,   -1, 2, 1 ], },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 3, 3, 2.5 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0, },
            "plane" : { "vertices" : [ -0.3, 1.99, -0.3,   0.3, 1.99, -0.3,   0.3, 1.99, 0.3,   -0.3, 1.99, 0.3 ], },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 0.5, 1.5, 0.5 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0.2, },
            "transform" : {
               "translate" : [ 0.6, 0.6, -0.5 ],
               "rotate" : [ 0, 0, 0,  0, 0, 1,  90 ],
               "triangle" : { "vertices" : [ 0, 0, 0,   0, 0, 0.4,   0.4, 0, 0 ],
                              "uvs" : [ 0, 0,   1, 0,   0, 1 ], },
            },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 2, 0.6, 0.4 ], },
            "bsdf" : { "type" : "diffuse", "kd" : 0.3, },
            "transform" : {
               "translate" : [ -0.4, 0.35, 0.2 ],
               "scale" : [ 0.25, 0.25, 0.25 ],
               "mesh" : { "path" : "octahedron.obj", },
            },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 1, 1, 1 ], },
            "transform" : {
               "translate" : [ 0.99, 1.0, 0 ],
               "rotate" : [ 0, 0, 0,  0, 0, 1,  90 ],
               "scale" : [ 0.5, 1, 0.5 ],
               "plane" : { },
            },
         },
      },
   },
}
